// boss_dist.cu -- exact output probabilities under particle losses, all outcomes at once.
//
// theboss's BSDistributionCalculatorWithFixedLosses
// (bs_distribution_calculator_with_fixed_losses.py:84-151) computes, for every
// outcome T with l particles, a sum over the distinct l-particle sub-occupations
// S' of the initial state ("lossy inputs", in the order
// generate_lossy_n_particle_input_states gives them,
// boson_sampling_utilities.py:158-203):
//     p(T) = [ sum_S' |perm(U[T, S'])|^2 / prod_i S'_i! * mult(S') ] / l! / C(n, l) * l! / prod_i T_i!
// with mult(S') = prod_i C(S_i, S_i - S'_i); theboss evaluates one outcome at a
// time (the uniform-loss calculator maps outcomes over a process pool,
// bs_exact_distribution_with_uniform_losses.py:62-71).  Here every (lossy input,
// outcome) pair of a particle count l is one GPU thread:
//   * lossy_pair_kernel<L> (L = l <= kDistMaxL): the Glynn permanent of the L x L
//     matrix (rows: the outcome's particles, columns: the lossy input's particles)
//     over the 2^(L-1) sign vectors with the first column's sign fixed, in
//     registers, then |perm|^2, theboss's divisions and the multiplicity;
//   * lossy_outcome_kernel: per outcome, the sum over lossy inputs in theboss's
//     order and the normalisation, with theboss's operation order.
// Larger l goes through the sweep engine (one Glynn sweep per pair, many threads
// each), and the same host arithmetic.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/boss.h"
#include "boss_internal.h"

namespace boss {

extern std::mutex g_api_mutex;

constexpr int kDistMaxL = 10;  // per-thread permanents up to 10 x 10 (512 sign vectors)
constexpr int kDistMaxDiv = 8;  // divisors (factorials of occupations >= 2) kept per state

// perm(U[rows, cols]) for one L x L matrix: Glynn's formula with the sign of
// column 0 fixed, columns 1..L-1 walked in binary-reflected Gray order.
template <int L>
__device__ __forceinline__ double2 glynn_small(const double2* __restrict__ U, int m, const int (&row)[L],
                                              const int (&col)[L]) {
  double sr[L], si[L];
#pragma unroll
  for (int a = 0; a < L; ++a) {
    double x = 0.0, y = 0.0;
#pragma unroll
    for (int b = 0; b < L; ++b) {
      const double2 u = U[(size_t)row[a] * m + col[b]];
      x += u.x;
      y += u.y;
    }
    sr[a] = x;
    si[a] = y;
  }
  double accr = 0.0, acci = 0.0;
  uint32_t neg = 0;  // bit b: column b currently has sign -1
  const uint32_t codes = 1u << (L - 1);
  for (uint32_t t = 0;;) {
    double pr = sr[0], pi = si[0];
#pragma unroll
    for (int a = 1; a < L; ++a) {
      const double r = fma(pr, sr[a], -(pi * si[a]));
      const double i = fma(pr, si[a], pi * sr[a]);
      pr = r;
      pi = i;
    }
    if (__popc(neg) & 1) {
      accr -= pr;
      acci -= pi;
    } else {
      accr += pr;
      acci += pi;
    }
    if (++t >= codes) break;
    const int b = __ffs(t);  // column 1 + ctz(t)
    const double c = ((neg >> b) & 1u) ? 2.0 : -2.0;
    neg ^= 1u << b;
#pragma unroll
    for (int a = 0; a < L; ++a) {
      const double2 u = U[(size_t)row[a] * m + col[b]];
      sr[a] = fma(c, u.x, sr[a]);
      si[a] = fma(c, u.y, si[a]);
    }
  }
  const double s = ldexp(1.0, -(L - 1));
  return make_double2(accr * s, acci * s);
}

template <int L>
__device__ __forceinline__ double glynn_abs2(const double2* __restrict__ U, int m, const int (&row)[L],
                                            const int (&col)[L]) {
  const double2 p = glynn_small<L>(U, m, row, col);
  return fma(p.x, p.x, p.y * p.y);
}

// Small permanents, one thread each: perm(U[T_k, S_k]) from the occupation rows
// (len entries, uint8) of equally many (L) input and output particles.
template <int L>
__global__ void __launch_bounds__(128) small_perm_kernel(const double2* __restrict__ U, int m, int len,
                                                         const uint8_t* __restrict__ S, const uint8_t* __restrict__ T,
                                                         int64_t count, double2* __restrict__ out) {
  const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= count) return;
  int row[L], col[L];
  int a = 0, b = 0;
  for (int i = 0; i < len; ++i) {
    for (int c = T[k * len + i]; c > 0 && a < L; --c) row[a++] = i;
    for (int c = S[k * len + i]; c > 0 && b < L; --c) col[b++] = i;
  }
  out[k] = glynn_small<L>(U, m, row, col);
}

// One thread per (lossy input k, outcome o); the layout [k][o] lets the outcome
// kernel read coalesced.
template <int L>
__global__ void __launch_bounds__(128) lossy_pair_kernel(const double2* __restrict__ U, int m,
                                                         const uint8_t* __restrict__ in_cols,  // [K][L]
                                                         const double* __restrict__ in_div,    // [K][kDistMaxDiv]
                                                         const int* __restrict__ in_ndiv,      // [K]
                                                         const double* __restrict__ in_mult,   // [K]
                                                         int K, const uint8_t* __restrict__ out_occ,  // [O][m]
                                                         int64_t O, double* __restrict__ terms) {     // [K][O]
  const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (int64_t)K * O) return;
  const int k = (int)(idx / O);
  const int64_t o = idx - (int64_t)k * O;
  int row[L], col[L];
#pragma unroll
  for (int a = 0; a < L; ++a) col[a] = in_cols[(size_t)k * L + a];
  {  // the outcome's particles, in mode order
    const uint8_t* occ = out_occ + o * m;
    int a = 0;
    for (int i = 0; i < m && a < L; ++i)
      for (int c = occ[i]; c > 0 && a < L; --c) row[a++] = i;
  }
  double v = glynn_abs2<L>(U, m, row, col);
  // bs_distribution_calculator_with_fixed_losses.py:137-142, same operation order
  const int nd = in_ndiv[k];
  for (int d = 0; d < nd; ++d) v /= in_div[(size_t)k * kDistMaxDiv + d];
  terms[idx] = v * in_mult[k];
}

__global__ void lossy_outcome_kernel(const double* __restrict__ terms, int K, int64_t O, int m,
                                     const uint8_t* __restrict__ out_occ,  // [O][m]
                                     const double* __restrict__ fact,      // [256] k! as theboss divides by it
                                     double fact_l, double binom_nl, double* __restrict__ prob) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= O) return;
  double p = 0.0;
  for (int k = 0; k < K; ++k) p += terms[(size_t)k * O + o];
  // bs_distribution_calculator_with_fixed_losses.py:145-149 and 99-104
  p /= fact_l;
  p /= binom_nl;
  p *= fact_l;
  const uint8_t* occ = out_occ + o * m;
  for (int i = 0; i < m; ++i)
    if (occ[i] >= 2) p /= fact[occ[i]];
  prob[o] = p;
}

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
static double factorial_d(int k) {  // exact up to 20!, then the nearest double of the product
  if (k <= 20) {
    uint64_t f = 1;
    for (int i = 2; i <= k; ++i) f *= (uint64_t)i;
    return (double)f;
  }
  long double f = 1.0L;
  for (int i = 2; i <= k; ++i) f *= (long double)i;
  return (double)f;
}

static double binom_d(int n, int k) {  // exact below 2^64
  if (k < 0 || k > n) return 0.0;
  k = std::min(k, n - k);
  unsigned __int128 c = 1;
  for (int i = 1; i <= k; ++i) c = c * (unsigned)(n - k + i) / (unsigned)i;
  return (double)c;
}

struct LossyInputs {
  std::vector<std::vector<int32_t>> occ;  // distinct sub-occupations, theboss's order
  std::vector<double> mult;               // prod_i C(S_i, S_i - S'_i)
};

// generate_lossy_n_particle_input_states (boson_sampling_utilities.py:175-203):
// combinations of particle indices in lexicographic order, first occurrence kept.
static int lossy_inputs(const int32_t* S, int m, int l, LossyInputs& out) {
  std::vector<int> x0;
  for (int i = 0; i < m; ++i)
    for (int c = 0; c < S[i]; ++c) x0.push_back(i);
  const int n = (int)x0.size();
  out.occ.clear();
  out.mult.clear();
  if (n == 0) {
    out.occ.push_back(std::vector<int32_t>(S, S + m));
    out.mult.push_back(1.0);
    return kOk;
  }
  if (l > n) return kOk;
  if (binom_d(n, l) > 5e7) {
    set_error("too many lossy input combinations (C(n, l) > 5e7)");
    return kErrLimit;
  }
  std::unordered_map<std::string, int> seen;
  std::vector<int> c(l);
  for (int i = 0; i < l; ++i) c[i] = i;
  std::vector<int32_t> occ(m);
  for (;;) {
    std::fill(occ.begin(), occ.end(), 0);
    for (int i = 0; i < l; ++i) occ[x0[c[i]]]++;
    std::string key((const char*)occ.data(), sizeof(int32_t) * m);
    if (seen.emplace(key, (int)out.occ.size()).second) {
      double mu = 1.0;  // bs_distribution_calculator_with_fixed_losses.py:162-169
      for (int i = 0; i < m; ++i) mu *= binom_d(S[i], S[i] - occ[i]);
      out.occ.push_back(occ);
      out.mult.push_back((double)(int64_t)mu);
    }
    int i = l - 1;
    while (i >= 0 && c[i] == n - l + i) --i;
    if (i < 0) break;
    c[i]++;
    for (int j = i + 1; j < l; ++j) c[j] = c[j - 1] + 1;
  }
  return kOk;
}

// Factorials of the occupations >= 2, in mode order (theboss divides by every
// factorial; those of 0 and 1 leave the value unchanged).
static int divisors(const int32_t* occ, int m, double* div) {
  int nd = 0;
  for (int i = 0; i < m; ++i)
    if (occ[i] >= 2) {
      if (nd == kDistMaxDiv) return -1;
      div[nd++] = factorial_d(occ[i]);
    }
  return nd;
}

static void particle_list(const int32_t* occ, int m, uint8_t* out) {
  int p = 0;
  for (int i = 0; i < m; ++i)
    for (int c = 0; c < occ[i]; ++c) out[p++] = (uint8_t)i;
}

template <int L>
static cudaError_t launch_pairs(const double2* U, int m, const uint8_t* cols, const double* div, const int* ndiv,
                                const double* mult, int K, const uint8_t* rows, int64_t O, double* terms,
                                cudaStream_t s) {
  const int64_t n = (int64_t)K * O;
  lossy_pair_kernel<L><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(U, m, cols, div, ndiv, mult, K, rows, O, terms);
  return cudaGetLastError();
}

static cudaError_t launch_pairs_l(int l, const double2* U, int m, const uint8_t* cols, const double* div,
                                  const int* ndiv, const double* mult, int K, const uint8_t* rows, int64_t O,
                                  double* terms, cudaStream_t s) {
  switch (l) {
    case 1: return launch_pairs<1>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 2: return launch_pairs<2>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 3: return launch_pairs<3>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 4: return launch_pairs<4>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 5: return launch_pairs<5>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 6: return launch_pairs<6>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 7: return launch_pairs<7>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 8: return launch_pairs<8>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 9: return launch_pairs<9>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    case 10: return launch_pairs<10>(U, m, cols, div, ndiv, mult, K, rows, O, terms, s);
    default: return cudaErrorInvalidValue;
  }
}

// All outcomes of one particle count l (1 <= l <= kDistMaxL) on the per-thread path.
static int group_small(Context* cx, const double* matrix, int m, int n, int l, const LossyInputs& LI,
                       const std::vector<const int32_t*>& outs, double* prob_out, const std::vector<int>& where,
                       float* kernel_ms) {
  const int K = (int)LI.occ.size();
  const int64_t O = (int64_t)outs.size();
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off = 0;
  const size_t o_U = off; off = al(off + sizeof(double2) * (size_t)m * m);
  const size_t o_fact = off; off = al(off + sizeof(double) * 256);
  const size_t o_cols = off; off = al(off + (size_t)K * l);
  const size_t o_div = off; off = al(off + sizeof(double) * (size_t)K * kDistMaxDiv);
  const size_t o_ndiv = off; off = al(off + sizeof(int) * (size_t)K);
  const size_t o_mult = off; off = al(off + sizeof(double) * (size_t)K);
  const size_t o_occ = off; off = al(off + (size_t)O * m);
  const size_t arena = off;
  int st;
  if ((st = ensure(cx->dist[0], arena))) return st;
  if ((st = ensure(cx->dist[1], sizeof(double) * (size_t)K * O))) return st;  // terms
  if ((st = ensure(cx->dist[2], sizeof(double) * (size_t)O))) return st;      // probabilities
  if ((st = ensure_pinned(cx, std::max(arena, sizeof(double) * (size_t)O)))) return st;
  char* h = (char*)cx->pinned;
  memcpy(h + o_U, matrix, sizeof(double2) * (size_t)m * m);
  double* hf = (double*)(h + o_fact);
  for (int k = 0; k < 256; ++k) hf[k] = factorial_d(k);
  for (int k = 0; k < K; ++k) {
    particle_list(LI.occ[k].data(), m, (uint8_t*)(h + o_cols) + (size_t)k * l);
    const int nd = divisors(LI.occ[k].data(), m, (double*)(h + o_div) + (size_t)k * kDistMaxDiv);
    if (nd < 0) {
      set_error("too many multiply occupied modes in a lossy input");
      return kErrLimit;
    }
    ((int*)(h + o_ndiv))[k] = nd;
    ((double*)(h + o_mult))[k] = LI.mult[k];
  }
  uint8_t* hocc = (uint8_t*)(h + o_occ);
  for (int64_t o = 0; o < O; ++o)
    for (int i = 0; i < m; ++i) hocc[(size_t)o * m + i] = (uint8_t)outs[o][i];
  char* d = (char*)cx->dist[0].ptr;
  double* terms = (double*)cx->dist[1].ptr;
  double* prob = (double*)cx->dist[2].ptr;
  cudaStream_t s = cx->stream;
  cudaError_t e = cudaMemcpyAsync(d, h, arena, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D distribution tables");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (kernel_ms) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s);
  }
  e = launch_pairs_l(l, (const double2*)(d + o_U), m, (const uint8_t*)(d + o_cols), (const double*)(d + o_div),
                     (const int*)(d + o_ndiv), (const double*)(d + o_mult), K, (const uint8_t*)(d + o_occ), O,
                     terms, s);
  if (e != cudaSuccess) return fail_cuda(e, "lossy pair kernel");
  lossy_outcome_kernel<<<(unsigned)((O + 127) / 128), 128, 0, s>>>(terms, K, O, m, (const uint8_t*)(d + o_occ),
                                                                   (const double*)(d + o_fact), factorial_d(l),
                                                                   binom_d(n, l), prob);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "lossy outcome kernel");
  if (kernel_ms) cudaEventRecord(e1, s);
  e = cudaMemcpyAsync(h, prob, sizeof(double) * (size_t)O, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return fail_cuda(e, "D2H probabilities");
  if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return fail_cuda(e, "distribution kernels");
  if (kernel_ms) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    *kernel_ms += ms;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
  }
  const double* hp = (const double*)h;
  for (int64_t o = 0; o < O; ++o) prob_out[where[o]] = hp[o];
  return kOk;
}

// Larger l: one Glynn sweep per (lossy input, outcome) on the sweep engine, the
// same arithmetic on the host.
static int group_large(Context* cx, const double* matrix, int m, int n, int l, const LossyInputs& LI,
                       const std::vector<const int32_t*>& outs, double* prob_out, const std::vector<int>& where) {
  const int K = (int)LI.occ.size();
  const int O = (int)outs.size();
  std::vector<double> terms((size_t)K * O, 0.0);
  std::vector<HostSweep> by_nf[kMaxFactors + 1];
  std::vector<size_t> which[kMaxFactors + 1];
  for (int k = 0; k < K; ++k)
    for (int o = 0; o < O; ++o) {
      HostSweep hs;
      bool need = false;
      double2 v = make_double2(0.0, 0.0);
      const int st = plan_permanent(matrix, m, LI.occ[k].data(), outs[o], m, BOSS_GLYNN, hs, need, v);
      if (st) return st;
      const size_t t = (size_t)k * O + o;
      if (need) {
        which[hs.nf].push_back(t);
        by_nf[hs.nf].push_back(std::move(hs));
      } else {
        terms[t] = v.x * v.x + v.y * v.y;
      }
    }
  for (int nf = 1; nf <= kMaxFactors; ++nf) {
    if (by_nf[nf].empty()) continue;
    std::vector<double2> res(by_nf[nf].size());
    const int st = run_sweeps(cx, by_nf[nf], false, 1, res.data());
    if (st) return st;
    for (size_t a = 0; a < res.size(); ++a) terms[which[nf][a]] = fma(res[a].x, res[a].x, res[a].y * res[a].y);
  }
  double div[kDistMaxDiv];
  for (int k = 0; k < K; ++k) {
    const int nd = divisors(LI.occ[k].data(), m, div);
    if (nd < 0) {
      set_error("too many multiply occupied modes in a lossy input");
      return kErrLimit;
    }
    for (int o = 0; o < O; ++o) {
      double v = terms[(size_t)k * O + o];
      for (int d = 0; d < nd; ++d) v /= div[d];
      terms[(size_t)k * O + o] = v * LI.mult[k];
    }
  }
  const double fl = factorial_d(l), bn = binom_d(n, l);
  for (int o = 0; o < O; ++o) {
    double p = 0.0;
    for (int k = 0; k < K; ++k) p += terms[(size_t)k * O + o];
    p /= fl;
    p /= bn;
    p *= fl;
    const int nd = divisors(outs[o], m, div);
    if (nd < 0) {
      set_error("too many multiply occupied modes in an outcome");
      return kErrLimit;
    }
    for (int d = 0; d < nd; ++d) p /= div[d];
    prob_out[where[o]] = p;
  }
  return kOk;
}

template <int L>
static cudaError_t launch_small(const double2* U, int m, int len, const uint8_t* S, const uint8_t* T, int64_t count,
                                double2* out, cudaStream_t s) {
  small_perm_kernel<L><<<(unsigned)((count + 127) / 128), 128, 0, s>>>(U, m, len, S, T, count, out);
  return cudaGetLastError();
}

static cudaError_t launch_small_l(int l, const double2* U, int m, int len, const uint8_t* S, const uint8_t* T,
                                  int64_t count, double2* out, cudaStream_t s) {
  switch (l) {
    case 1: return launch_small<1>(U, m, len, S, T, count, out, s);
    case 2: return launch_small<2>(U, m, len, S, T, count, out, s);
    case 3: return launch_small<3>(U, m, len, S, T, count, out, s);
    case 4: return launch_small<4>(U, m, len, S, T, count, out, s);
    case 5: return launch_small<5>(U, m, len, S, T, count, out, s);
    case 6: return launch_small<6>(U, m, len, S, T, count, out, s);
    case 7: return launch_small<7>(U, m, len, S, T, count, out, s);
    case 8: return launch_small<8>(U, m, len, S, T, count, out, s);
    case 9: return launch_small<9>(U, m, len, S, T, count, out, s);
    case 10: return launch_small<10>(U, m, len, S, T, count, out, s);
    default: return cudaErrorInvalidValue;
  }
}

int small_perm_batch(Context* cx, const double* matrix, int m, int len, const int32_t* S, const int32_t* T,
                     const std::vector<int>* by_l, double2* results) {
  int64_t total = 0;
  for (int l = 1; l <= kSmallPermMax; ++l) total += (int64_t)by_l[l].size();
  if (total == 0) return kOk;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t o_U = 0, o_S = al(sizeof(double2) * (size_t)m * m), o_T = o_S + al((size_t)total * len);
  const size_t o_out = o_T + al((size_t)total * len), arena = o_out + sizeof(double2) * (size_t)total;
  int st;
  if ((st = ensure(cx->dist[3], arena))) return st;
  if ((st = ensure_pinned(cx, arena))) return st;
  char* h = (char*)cx->pinned;
  memcpy(h + o_U, matrix, sizeof(double2) * (size_t)m * m);
  uint8_t* hS = (uint8_t*)(h + o_S);
  uint8_t* hT = (uint8_t*)(h + o_T);
  int64_t at = 0;
  for (int l = 1; l <= kSmallPermMax; ++l)
    for (int k : by_l[l]) {
      for (int i = 0; i < len; ++i) {
        hS[at * len + i] = (uint8_t)S[(size_t)k * len + i];
        hT[at * len + i] = (uint8_t)T[(size_t)k * len + i];
      }
      ++at;
    }
  char* d = (char*)cx->dist[3].ptr;
  cudaStream_t s = cx->stream;
  cudaError_t e = cudaMemcpyAsync(d, h, o_out, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D small permanents");
  at = 0;
  for (int l = 1; l <= kSmallPermMax; ++l) {
    const int64_t c = (int64_t)by_l[l].size();
    if (!c) continue;
    e = launch_small_l(l, (const double2*)(d + o_U), m, len, (const uint8_t*)(d + o_S) + at * len,
                       (const uint8_t*)(d + o_T) + at * len, c, (double2*)(d + o_out) + at, s);
    if (e != cudaSuccess) return fail_cuda(e, "small permanents");
    at += c;
  }
  e = cudaMemcpyAsync(h + o_out, d + o_out, sizeof(double2) * (size_t)total, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail_cuda(e, "small permanents");
  const double2* hr = (const double2*)(h + o_out);
  at = 0;
  for (int l = 1; l <= kSmallPermMax; ++l)
    for (int k : by_l[l]) results[k] = hr[at++];
  return kOk;
}

}  // namespace boss

using namespace boss;

extern "C" {

int boss_lossy_probabilities(const double* matrix, int32_t m, const int32_t* initial_state, const int32_t* outcomes,
                             int32_t count, double* probabilities, float* kernel_ms) {
  if (!matrix || !initial_state || (count > 0 && (!outcomes || !probabilities)) || m <= 0 || count < 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (m > 256) {
    set_error("at most 256 modes");
    return kErrLimit;
  }
  int n = 0;
  for (int i = 0; i < m; ++i) {
    if (initial_state[i] < 0 || initial_state[i] > 255) {
      set_error("occupations must be in [0, 255]");
      return kErrArg;
    }
    n += initial_state[i];
  }
  if (n > 255) {
    set_error("at most 255 input particles");
    return kErrLimit;
  }
  if (kernel_ms) *kernel_ms = 0.f;
  std::lock_guard<std::mutex> lk(g_api_mutex);
  // group the outcomes by particle count
  std::vector<std::vector<const int32_t*>> by_l(n + 1);
  std::vector<std::vector<int>> where(n + 1);
  for (int o = 0; o < count; ++o) {
    const int32_t* T = outcomes + (size_t)o * m;
    int l = 0;
    for (int i = 0; i < m; ++i) {
      if (T[i] < 0 || T[i] > 255) {
        set_error("occupations must be in [0, 255]");
        return kErrArg;
      }
      l += T[i];
    }
    if (l > n) {
      set_error("an outcome holds more particles than the initial state");
      return kErrArg;
    }
    if (l == 0) {  // the empty lossy input: perm = 1, every factor 1
      probabilities[o] = 1.0;
      continue;
    }
    by_l[l].push_back(T);
    where[l].push_back(o);
  }
  int st;
  Context* cx = nullptr;
  for (int l = 1; l <= n; ++l) {
    if (by_l[l].empty()) continue;
    if (!cx && !(cx = context(&st))) return st;
    LossyInputs LI;
    if ((st = lossy_inputs(initial_state, m, l, LI))) return st;
    st = (l <= kDistMaxL) ? group_small(cx, matrix, m, n, l, LI, by_l[l], probabilities, where[l], kernel_ms)
                          : group_large(cx, matrix, m, n, l, LI, by_l[l], probabilities, where[l]);
    if (st) return st;
  }
  return kOk;
}

}  // extern "C"
