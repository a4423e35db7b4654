// boss_count.cu -- frequencies of sampled outcomes.
//
// theboss's BSSampleBasedDistributionCalculator
// (bs_sample_based_distribution_calculator.py:74-110) compares every sample with
// every listed outcome in Python (O(samples x outcomes)) and counts it for the
// first outcome equal to it.  Here the outcomes go into a device hash table
// (open addressing, linear probing, full-key comparison; equal outcomes keep the
// smallest index, so the first listed one receives the counts) and every sample
// is one lookup plus an integer atomic add: counts are exact and independent of
// the order the GPU runs the threads in.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/boss.h"
#include "boss_internal.h"

namespace boss {

extern std::mutex g_api_mutex;

__device__ __forceinline__ uint64_t state_hash(const uint8_t* s, int m) {
  uint64_t h = 1469598103934665603ull;  // FNV-1a
  for (int i = 0; i < m; ++i) h = (h ^ s[i]) * 1099511628211ull;
  return h ^ (h >> 29);
}

__device__ __forceinline__ bool state_equal(const uint8_t* a, const uint8_t* b, int m) {
  for (int i = 0; i < m; ++i)
    if (a[i] != b[i]) return false;
  return true;
}

__global__ void outcome_insert_kernel(const uint8_t* __restrict__ outcomes, int64_t O, int m, int* table,
                                      uint64_t mask) {
  const int64_t o = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= O) return;
  const uint8_t* key = outcomes + o * m;
  uint64_t slot = state_hash(key, m) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe, slot = (slot + 1) & mask) {
    const int prev = atomicCAS(&table[slot], -1, (int)o);
    if (prev == -1) return;
    if (state_equal(outcomes + (int64_t)prev * m, key, m)) {  // the same outcome listed twice
      atomicMin(&table[slot], (int)o);
      return;
    }
  }
}

__global__ void outcome_count_kernel(const uint8_t* __restrict__ samples, int64_t S, int m,
                                     const uint8_t* __restrict__ outcomes, const int* __restrict__ table,
                                     uint64_t mask, unsigned long long* counts) {
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= S) return;
  const uint8_t* key = samples + s * m;
  uint64_t slot = state_hash(key, m) & mask;
  for (uint64_t probe = 0; probe <= mask; ++probe, slot = (slot + 1) & mask) {
    const int o = table[slot];
    if (o < 0) return;  // not a listed outcome
    if (state_equal(outcomes + (int64_t)o * m, key, m)) {
      atomicAdd(&counts[o], 1ull);
      return;
    }
  }
}

}  // namespace boss

using namespace boss;

extern "C" {

int boss_count_outcomes(const int32_t* samples, int64_t n_samples, const int32_t* outcomes, int64_t n_outcomes,
                        int32_t m, int64_t* counts) {
  if (m <= 0 || n_samples < 0 || n_outcomes < 0 || (n_samples > 0 && !samples) ||
      (n_outcomes > 0 && (!outcomes || !counts))) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (n_outcomes > (int64_t)1 << 30) {
    set_error("at most 2^30 outcomes");
    return kErrLimit;
  }
  std::fill(counts, counts + n_outcomes, (int64_t)0);
  if (n_outcomes == 0 || n_samples == 0) return kOk;
  std::lock_guard<std::mutex> lk(g_api_mutex);
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  uint64_t tsize = 1024;
  while (tsize < 2 * (uint64_t)n_outcomes) tsize <<= 1;
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  const size_t b_out = al((size_t)n_outcomes * m), b_smp = al((size_t)n_samples * m);
  const size_t o_out = 0, o_smp = b_out, arena = b_out + b_smp;
  if ((st = ensure(cx->dist[0], arena))) return st;
  if ((st = ensure(cx->dist[1], sizeof(int) * tsize))) return st;
  if ((st = ensure(cx->dist[2], sizeof(unsigned long long) * (size_t)n_outcomes))) return st;
  if ((st = ensure_pinned(cx, std::max(arena, sizeof(unsigned long long) * (size_t)n_outcomes)))) return st;
  uint8_t* h = (uint8_t*)cx->pinned;
  // States as bytes; an entry outside [0, 255] cannot be sampled, so such an
  // outcome gets an impossible key (all 0xff) and such a sample is rejected.
  for (int64_t o = 0; o < n_outcomes; ++o) {
    bool ok = true;
    for (int i = 0; i < m; ++i) ok &= (outcomes[o * m + i] >= 0 && outcomes[o * m + i] < 255);
    for (int i = 0; i < m; ++i) h[o_out + o * m + i] = ok ? (uint8_t)outcomes[o * m + i] : 0xff;
  }
  for (int64_t s = 0; s < n_samples; ++s)
    for (int i = 0; i < m; ++i) {
      const int32_t v = samples[s * m + i];
      if (v < 0 || v >= 255) {
        set_error("sample occupations must be in [0, 254]");
        return kErrArg;
      }
      h[o_smp + s * m + i] = (uint8_t)v;
    }
  cudaStream_t strm = cx->stream;
  uint8_t* d = (uint8_t*)cx->dist[0].ptr;
  int* table = (int*)cx->dist[1].ptr;
  unsigned long long* dc = (unsigned long long*)cx->dist[2].ptr;
  cudaError_t e = cudaMemcpyAsync(d, h, arena, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess) e = cudaMemsetAsync(table, 0xff, sizeof(int) * tsize, strm);
  if (e == cudaSuccess) e = cudaMemsetAsync(dc, 0, sizeof(unsigned long long) * (size_t)n_outcomes, strm);
  if (e != cudaSuccess) return fail_cuda(e, "outcome table upload");
  outcome_insert_kernel<<<(unsigned)((n_outcomes + 255) / 256), 256, 0, strm>>>(d + o_out, n_outcomes, m, table,
                                                                                tsize - 1);
  outcome_count_kernel<<<(unsigned)((n_samples + 255) / 256), 256, 0, strm>>>(d + o_smp, n_samples, m, d + o_out,
                                                                              table, tsize - 1, dc);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "outcome counting");
  e = cudaMemcpyAsync(h, dc, sizeof(unsigned long long) * (size_t)n_outcomes, cudaMemcpyDeviceToHost, strm);
  if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
  if (e != cudaSuccess) return fail_cuda(e, "outcome counting");
  memcpy(counts, h, sizeof(int64_t) * (size_t)n_outcomes);
  return kOk;
}

}  // extern "C"
