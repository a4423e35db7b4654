// boss_perm.cu -- dispatch of the NF-templated sweep kernels, the fixed-order
// reductions of their partials, and the thread partition shared by every caller.
#include <algorithm>
#include <cmath>

#include "boss_internal.h"

namespace boss {

cudaError_t sweep_nf_a_launch(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st);
cudaError_t sweep_nf_b_launch(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st);
cudaError_t sweep_nf_c_launch(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st);
cudaError_t sweep_nf_d_launch(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st);
cudaError_t sweep_nf_a_prepare(int* perm_occ, int* minors_occ, int* ff_occ, int* pff_occ);
cudaError_t sweep_nf_b_prepare(int* perm_occ, int* minors_occ, int* ff_occ, int* pff_occ);
cudaError_t sweep_nf_c_prepare(int* perm_occ, int* minors_occ, int* ff_occ, int* pff_occ);
cudaError_t sweep_nf_d_prepare(int* perm_occ, int* minors_occ, int* ff_occ, int* pff_occ);

cudaError_t sweep_nf_a_grad_occupancy(int nf, int* occ);
cudaError_t sweep_nf_b_grad_occupancy(int nf, int* occ);
cudaError_t sweep_nf_c_grad_occupancy(int nf, int* occ);
cudaError_t sweep_nf_d_grad_occupancy(int nf, int* occ);

static int g_perm_occ[kMaxFactors + 1];
static int g_perm_ff_occ[kMaxFactors + 1];
static int g_minors_occ[kMaxFactors + 1][kMaxMinorDigits + 1];     // [nf][rows of minors]
static int g_minors_ff_occ[kMaxFactors + 1][kMaxMinorDigits + 1];  // float-pair kernel; 0: none

cudaError_t prepare_sweep_kernels() {
  cudaError_t e;
  if ((e = sweep_nf_a_prepare(g_perm_occ + 1, &g_minors_occ[1][0], &g_minors_ff_occ[1][0], g_perm_ff_occ + 1)))
    return e;
  if ((e = sweep_nf_b_prepare(g_perm_occ + 9, &g_minors_occ[9][0], &g_minors_ff_occ[9][0], g_perm_ff_occ + 9)))
    return e;
  if ((e = sweep_nf_c_prepare(g_perm_occ + 17, &g_minors_occ[17][0], &g_minors_ff_occ[17][0], g_perm_ff_occ + 17)))
    return e;
  return sweep_nf_d_prepare(g_perm_occ + 25, &g_minors_occ[25][0], &g_minors_ff_occ[25][0], g_perm_ff_occ + 25);
}

bool perm_ff_available(int nf) { return nf >= 1 && nf <= kMaxFactors && g_perm_ff_occ[nf] > 0; }

bool minors_ff_available(int nf) { return nf >= 1 && nf <= kMaxFactors && g_minors_ff_occ[nf][kMaxMinorDigits] > 0; }

int64_t sweep_resident_minors(int nf, int rows, int sm_count, bool ff) {
  if (nf < 1 || nf > kMaxFactors) return 128;
  rows = std::min(std::max(rows, 1), kMaxMinorDigits);
  const int occ = ff ? g_minors_ff_occ[nf][rows] : g_minors_occ[nf][rows];
  return (int64_t)std::max(1, occ) * sm_count * 128;
}

int64_t sweep_resident_threads(int nf, SweepOp op, int sm_count) {
  if (nf < 1 || nf > kMaxFactors) return 128;
  if (op == SweepOp::kGrad) {
    int occ = 1;
    cudaError_t e = (nf <= 8)    ? sweep_nf_a_grad_occupancy(nf, &occ)
                    : (nf <= 16) ? sweep_nf_b_grad_occupancy(nf, &occ)
                    : (nf <= 24) ? sweep_nf_c_grad_occupancy(nf, &occ)
                                 : sweep_nf_d_grad_occupancy(nf, &occ);
    if (e != cudaSuccess) {
      cudaGetLastError();
      occ = 1;
    }
    return (int64_t)std::max(occ, 1) * sm_count * 64;
  }
  const int occ = std::max(1, op == SweepOp::kPerm     ? g_perm_occ[nf]
                              : op == SweepOp::kPermFF ? g_perm_ff_occ[nf]
                                                       : g_minors_occ[nf][kMaxMinorDigits]);
  return (int64_t)occ * sm_count * 128;
}

cudaError_t launch_sweep(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st) {
  if (L.total_threads <= 0) return cudaSuccess;
  if (nf >= 1 && nf <= 8) return sweep_nf_a_launch(nf, op, L, st);
  if (nf <= 16) return sweep_nf_b_launch(nf, op, L, st);
  if (nf <= 24) return sweep_nf_c_launch(nf, op, L, st);
  if (nf <= 32) return sweep_nf_d_launch(nf, op, L, st);
  return cudaErrorInvalidValue;
}

void partition_threads(const std::vector<uint64_t>& n_codes, int64_t resident, std::vector<int64_t>& n_threads) {
  const size_t n = n_codes.size();
  n_threads.assign(n, 1);
  long double total = 0;
  for (uint64_t c : n_codes) total += (long double)c;
  if (total <= 0) return;
  long double want = std::min<long double>((long double)resident, total / (long double)kMinCodesPerThread);
  want = std::max<long double>(want, (long double)n);
  for (size_t p = 0; p < n; ++p) {
    long double t = want * (long double)n_codes[p] / total;
    int64_t k = (int64_t)std::floor(t);
    k = std::max<int64_t>(k, 1);
    k = std::min<int64_t>(k, (int64_t)std::max<uint64_t>(n_codes[p], 1));
    n_threads[p] = k;
  }
}

// One block per sweep: fixed-order sum of its threads' partials.
// ff: the partials are float pairs (float4), as the float-pair sweep writes them.
__global__ void perm_reduce_kernel(const SweepProblem* __restrict__ probs, const double2* __restrict__ partials,
                                   double2* __restrict__ out, int ff) {
  __shared__ double sr[256], si[256];
  const SweepProblem& P = probs[blockIdx.x];
  double ar = 0.0, ai = 0.0;
  for (int64_t i = threadIdx.x; i < P.n_threads; i += blockDim.x) {
    double2 v;
    if (ff) {
      const float4 f = reinterpret_cast<const float4*>(partials)[P.part_off + i];
      v = make_double2(ff_to_double(f.x, f.y), ff_to_double(f.z, f.w));
    } else {
      v = partials[P.part_off + i];
    }
    ar += v.x;
    ai += v.y;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[P.out_idx] = make_double2(sr[0] * P.scale, si[0] * P.scale);
}

// One block per all-minors sweep; digit by digit, a fixed-order tree sum over the
// threads' partials.
// ff: the partials are float pairs (float4), as the float-pair sweep writes them.
__global__ void minors_reduce_kernel(const SweepProblem* __restrict__ probs, const double2* __restrict__ partials,
                                     double2* __restrict__ out, int nd_max, int ff) {
  __shared__ double sr[256], si[256];
  const SweepProblem& P = probs[blockIdx.x];
  const int nd = P.nd + P.fixed_digit;  // the held digit's row last
  for (int j = 0; j < nd; ++j) {
    double ar = 0.0, ai = 0.0;
    for (int64_t q = threadIdx.x; q < P.n_threads; q += blockDim.x) {
      double2 v;
      if (ff) {
        const float4 f = reinterpret_cast<const float4*>(partials)[P.part_off + q * nd + j];
        v = make_double2(ff_to_double(f.x, f.y), ff_to_double(f.z, f.w));
      } else {
        v = partials[P.part_off + q * nd + j];
      }
      ar += v.x;
      ai += v.y;
    }
    sr[threadIdx.x] = ar;
    si[threadIdx.x] = ai;
    __syncthreads();
    for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
      if ((int)threadIdx.x < s) {
        sr[threadIdx.x] += sr[threadIdx.x + s];
        si[threadIdx.x] += si[threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)P.out_idx * nd_max + j] = make_double2(sr[0] * P.scale, si[0] * P.scale);
    __syncthreads();
  }
}

// One block per gradient sweep: every (digit, factor) entry of the per-warp
// gradient partials and the per-warp permanents, summed over the sweep's groups
// of 32 threads in a fixed order.  grad_out row = (nd + fixed) x nf entries.
__global__ void grad_reduce_kernel(const SweepProblem* __restrict__ probs, const double2* __restrict__ gpart,
                                   const double2* __restrict__ ppart, double2* __restrict__ grad_out,
                                   double2* __restrict__ perm_out, int row_stride) {
  __shared__ double sr[256], si[256];
  const SweepProblem& P = probs[blockIdx.x];
  const int ne = (P.nd + P.fixed_digit) * P.nf;
  const int64_t groups = P.n_threads >> 5;  // each group of 32 threads left one compact partial
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    double ar = 0.0, ai = 0.0;
    for (int64_t g = 0; g < groups; ++g) {
      const double2 v = gpart[P.part_off + g * (int64_t)ne * 32 + e];
      ar += v.x;
      ai += v.y;
    }
    grad_out[(size_t)P.out_idx * row_stride + e] = make_double2(ar * P.scale, ai * P.scale);
  }
  double ar = 0.0, ai = 0.0;
  for (int64_t q = threadIdx.x; q < groups; q += blockDim.x) {
    const double2 v = ppart[(P.thread_begin >> 5) + q];
    ar += v.x;
    ai += v.y;
  }
  sr[threadIdx.x] = ar;
  si[threadIdx.x] = ai;
  __syncthreads();
  for (int s = blockDim.x >> 1; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      sr[threadIdx.x] += sr[threadIdx.x + s];
      si[threadIdx.x] += si[threadIdx.x + s];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) perm_out[P.out_idx] = make_double2(sr[0] * P.scale, si[0] * P.scale);
}

cudaError_t launch_grad_reduce(const SweepProblem* probs, int n_probs, const double2* gpart, const double2* ppart,
                               double2* grad_out, double2* perm_out, int row_stride, cudaStream_t st) {
  if (n_probs <= 0) return cudaSuccess;
  grad_reduce_kernel<<<n_probs, 256, 0, st>>>(probs, gpart, ppart, grad_out, perm_out, row_stride);
  return cudaGetLastError();
}

cudaError_t launch_perm_reduce(const SweepProblem* probs, int n_probs, const double2* partials, double2* out,
                               cudaStream_t st, bool ff) {
  if (n_probs <= 0) return cudaSuccess;
  perm_reduce_kernel<<<n_probs, 256, 0, st>>>(probs, partials, out, ff ? 1 : 0);
  return cudaGetLastError();
}

cudaError_t launch_minors_reduce(const SweepProblem* probs, int n_probs, const double2* partials, double2* out,
                                 int nd_max, cudaStream_t st, bool ff) {
  if (n_probs <= 0) return cudaSuccess;
  minors_reduce_kernel<<<n_probs, 256, 0, st>>>(probs, partials, out, nd_max, ff ? 1 : 0);
  return cudaGetLastError();
}

}  // namespace boss
