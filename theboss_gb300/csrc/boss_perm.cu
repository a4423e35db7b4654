// boss_perm.cu -- permanents and all-minors permanents on the GPU.
//
//   perm_sweep_kernel<NC>    : one warp = 32 chunks of one sweep segment; writes one
//                              complex partial per work item.
//   minors_sweep_kernel<NC>  : the all-minors (C&C-B) sweep of
//                              bs_cc_ryser_submatrices_permanent_calculator.py:73-119;
//                              writes nd complex partials per work item.
//   *_reduce_kernel          : fixed-order reduction of the partials (bit-identical
//                              results run to run).
//
// Work items are handed out by an atomic counter (one atomicAdd per warp per item),
// so big and small sweeps in one launch balance without a host-side schedule.
#include "boss_internal.h"

namespace boss {

// ---------------------------------------------------------------------------
// Kernels
// ---------------------------------------------------------------------------
__device__ __forceinline__ int find_plan(const SweepPlan* __restrict__ plans, int n_plans, int64_t item) {
  int lo = 0, hi = n_plans - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (plans[mid].item_off <= item) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ int64_t next_item(unsigned long long* counter, int lane) {
  unsigned long long it = 0;
  if (lane == 0) it = atomicAdd(counter, 1ull);
  return (int64_t)__shfl_sync(0xffffffffu, it, 0);
}

template <int NC>
__global__ void __launch_bounds__(128) perm_sweep_kernel(const SweepPlan* __restrict__ plans, int n_plans,
                                                         const double2* __restrict__ pool, int64_t total_items,
                                                         unsigned long long* __restrict__ counter,
                                                         double2* __restrict__ partials) {
  const int lane = threadIdx.x & 31;
  for (int64_t item = next_item(counter, lane); item < total_items; item = next_item(counter, lane)) {
    const SweepPlan& P = plans[find_plan(plans, n_plans, item)];
    const int64_t chunk = (item - P.item_off) * 32 + lane;
    double acc_r = 0.0, acc_i = 0.0;
    if (chunk < P.n_chunks) {
      const double2* D = pool + P.mat_off;
      const double2* base = pool + P.base_off;
      double sr[NC], si[NC];
      uint32_t parity, g;
      double w;
      const int c = P.c;
      decode_chunk_start<NC>(P, D, base, (uint64_t)P.code_off + ((uint64_t)chunk << c), sr, si, parity, w, g);
      double pr, pi;
      column_product<NC>(P, sr, si, pr, pi);
      acc_r = xor_sign(pr, parity << 31);
      acc_i = xor_sign(pi, parity << 31);
      const uint32_t n = 1u << c;
      for (uint32_t local = 1; local < n; ++local) {
        const int i = __ffs(local) - 1;
        const uint32_t bit = (g >> i) & 1u;
        g ^= 1u << i;
        flip_digit<NC>(P, D, i, bit, sr, si);
        parity ^= 1u;
        column_product<NC>(P, sr, si, pr, pi);
        acc_r += xor_sign(pr, parity << 31);
        acc_i += xor_sign(pi, parity << 31);
      }
      acc_r *= w;
      acc_i *= w;
    }
    acc_r = warp_sum(acc_r);
    acc_i = warp_sum(acc_i);
    if (lane == 0) partials[P.part_off + (item - P.item_off)] = make_double2(acc_r, acc_i);
  }
}

// One block per result: sums the partials of every segment of that result in a
// fixed order, then applies the segment scale (all segments of a result share it).
__global__ void perm_reduce_kernel(const SweepPlan* __restrict__ plans, const int32_t* __restrict__ out_plans,
                                   const int32_t* __restrict__ out_begin, const double2* __restrict__ partials,
                                   double2* __restrict__ out) {
  __shared__ double sr[256], si[256];
  const int o = blockIdx.x;
  const int p0 = out_begin[o], p1 = out_begin[o + 1];
  double ar = 0.0, ai = 0.0;
  for (int p = p0; p < p1; ++p) {
    const SweepPlan& P = plans[out_plans[p]];
    for (int64_t i = threadIdx.x; i < P.n_items; i += blockDim.x) {
      const double2 v = partials[P.part_off + i];
      ar += v.x;
      ai += v.y;
    }
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
  if (threadIdx.x == 0) {
    const double sc = (p1 > p0) ? plans[out_plans[p0]].scale : 1.0;
    out[o] = make_double2(sr[0] * sc, si[0] * sc);
  }
}

// Value of digit i in code t (closed form of the reflected mixed-radix code).
__device__ __forceinline__ uint32_t digit_value(const SweepPlan& P, uint64_t t, int i) {
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

// All-minors sweep (Ryser flavour).  For binary low digits the minor of digit i
// receives every code with r_i = 0.  Instead of adding each product into every
// such minor, a running signed total R of all products is kept, and each minor
// is settled only when its digit flips: a flip 0->1 ends a run of r_i = 0 codes
// (minor_i += R), a flip 1->0 starts one (minor_i -= R).  That is 4 DADD per code
// instead of one complex add per minor.  Digits that are constant over the chunk
// receive R times their weight (S_i - r_i) / S_i at the end.
// Dynamic shared memory: 16 rows x 32 lanes x double2 per warp.
template <int NC>
__global__ void __launch_bounds__(128) minors_sweep_kernel(const SweepPlan* __restrict__ plans, int n_plans,
                                                           const double2* __restrict__ pool, int64_t total_items,
                                                           unsigned long long* __restrict__ counter,
                                                           double2* __restrict__ partials) {
  extern __shared__ double2 stage_all[];
  const int lane = threadIdx.x & 31;
  double2* st = stage_all + (threadIdx.x >> 5) * (16 * 32);
  for (int64_t item = next_item(counter, lane); item < total_items; item = next_item(counter, lane)) {
    const SweepPlan& P = plans[find_plan(plans, n_plans, item)];
    const int64_t chunk = (item - P.item_off) * 32 + lane;
    const bool active = chunk < P.n_chunks;
    const int c = P.c;  // <= 16
    const int nd = P.nd;
    const uint64_t t0 = (uint64_t)P.code_off + ((uint64_t)(active ? chunk : 0) << c);
    for (int i = 0; i < c; ++i) st[i * 32 + lane] = make_double2(0.0, 0.0);
    double Rr = 0.0, Ri = 0.0, w = 0.0;
    uint32_t g = 0;
    if (active) {
      const double2* D = pool + P.mat_off;
      const double2* base = pool + P.base_off;
      double sr[NC], si[NC];
      uint32_t parity;
      decode_chunk_start<NC>(P, D, base, t0, sr, si, parity, w, g);
      double pr, pi;
      column_product<NC>(P, sr, si, pr, pi);
      Rr = xor_sign(pr, parity << 31);
      Ri = xor_sign(pi, parity << 31);
      const uint32_t n = 1u << c;
      for (uint32_t local = 1; local < n; ++local) {
        const int i = __ffs(local) - 1;
        const uint32_t bit = (g >> i) & 1u;
        double2 mv = st[i * 32 + lane];
        mv.x += xor_sign(Rr, bit << 31);
        mv.y += xor_sign(Ri, bit << 31);
        st[i * 32 + lane] = mv;
        g ^= 1u << i;
        flip_digit<NC>(P, D, i, bit, sr, si);
        parity ^= 1u;
        column_product<NC>(P, sr, si, pr, pi);
        Rr += xor_sign(pr, parity << 31);
        Ri += xor_sign(pi, parity << 31);
      }
      for (int i = 0; i < c; ++i) {
        if (((g >> i) & 1u) == 0u) {
          double2 mv = st[i * 32 + lane];
          mv.x += Rr;
          mv.y += Ri;
          st[i * 32 + lane] = mv;
        }
      }
    }
    // Settle every digit in groups of 16 rows: each lane writes its weighted value,
    // then lane j sums row j over the 32 lanes in lane order.
    const int64_t out_base = P.part_off + (item - P.item_off) * (int64_t)nd;
    for (int g0 = 0; g0 < nd; g0 += 16) {
      for (int j = 0; j < 16 && g0 + j < nd; ++j) {
        const int i = g0 + j;
        double2 v;
        if (!active) {
          v = make_double2(0.0, 0.0);
        } else if (i < c) {
          v = st[i * 32 + lane];
          v.x *= w;
          v.y *= w;
        } else {
          const uint32_t r = digit_value(P, t0, i);
          const uint32_t mu = P.mult[i];
          const double wi = (r < mu) ? w * ((double)(mu - r) / (double)mu) : 0.0;
          v = make_double2(Rr * wi, Ri * wi);
        }
        st[j * 32 + lane] = v;
      }
      __syncwarp();
      if (lane < 16 && g0 + lane < nd) {
        double sx = 0.0, sy = 0.0;
        for (int l = 0; l < 32; ++l) {
          const double2 v = st[lane * 32 + l];
          sx += v.x;
          sy += v.y;
        }
        partials[out_base + g0 + lane] = make_double2(sx, sy);
      }
      __syncwarp();
    }
  }
}

// One block per all-minors result; thread j < nd sums digit j over the items of
// every segment in a fixed order.  out row o holds nd_max complex entries.
__global__ void minors_reduce_kernel(const SweepPlan* __restrict__ plans, const int32_t* __restrict__ out_plans,
                                     const int32_t* __restrict__ out_begin, const double2* __restrict__ partials,
                                     double2* __restrict__ out, int nd_max) {
  const int o = blockIdx.x;
  const int p0 = out_begin[o], p1 = out_begin[o + 1];
  if (p1 <= p0) return;
  const int nd = plans[out_plans[p0]].nd;
  for (int j = threadIdx.x; j < nd; j += blockDim.x) {
    double sx = 0.0, sy = 0.0;
    for (int p = p0; p < p1; ++p) {
      const SweepPlan& P = plans[out_plans[p]];
      for (int64_t it = 0; it < P.n_items; ++it) {
        const double2 v = partials[P.part_off + it * nd + j];
        sx += v.x;
        sy += v.y;
      }
    }
    const double sc = plans[out_plans[p0]].scale;
    out[(size_t)o * nd_max + j] = make_double2(sx * sc, sy * sc);
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
template <int NC>
static cudaError_t launch_perm_nc(const SweepLaunch& L, cudaStream_t st) {
  perm_sweep_kernel<NC><<<L.grid, 128, 0, st>>>(L.plans, L.n_plans, L.pool, L.total_items, L.counter, L.partials);
  return cudaGetLastError();
}

constexpr size_t kMinorsSmem = 4 * 16 * 32 * sizeof(double2);

template <int NC>
static cudaError_t launch_minors_nc(const SweepLaunch& L, cudaStream_t st) {
  minors_sweep_kernel<NC><<<L.grid, 128, kMinorsSmem, st>>>(L.plans, L.n_plans, L.pool, L.total_items, L.counter,
                                                           L.partials);
  return cudaGetLastError();
}

// Kernel attributes are set once per process, outside any stream capture.
cudaError_t prepare_sweep_kernels() {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(minors_sweep_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kMinorsSmem)) != cudaSuccess)
    return e;
  if ((e = cudaFuncSetAttribute(minors_sweep_kernel<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)kMinorsSmem)) != cudaSuccess)
    return e;
  return cudaFuncSetAttribute(minors_sweep_kernel<32>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)kMinorsSmem);
}

cudaError_t launch_perm_sweep(const SweepLaunch& L, cudaStream_t st) {
  if (L.max_nc <= 8) return launch_perm_nc<8>(L, st);
  if (L.max_nc <= 16) return launch_perm_nc<16>(L, st);
  return launch_perm_nc<32>(L, st);
}

cudaError_t launch_minors_sweep(const SweepLaunch& L, cudaStream_t st) {
  if (L.max_nc <= 8) return launch_minors_nc<8>(L, st);
  if (L.max_nc <= 16) return launch_minors_nc<16>(L, st);
  return launch_minors_nc<32>(L, st);
}

cudaError_t launch_perm_reduce(const SweepPlan* plans, const int32_t* out_plans, const int32_t* out_begin, int n_out,
                               const double2* partials, double2* out, cudaStream_t st) {
  if (n_out <= 0) return cudaSuccess;
  perm_reduce_kernel<<<n_out, 256, 0, st>>>(plans, out_plans, out_begin, partials, out);
  return cudaGetLastError();
}

cudaError_t launch_minors_reduce(const SweepPlan* plans, const int32_t* out_plans, const int32_t* out_begin,
                                 int n_out, const double2* partials, double2* out, int nd_max, cudaStream_t st) {
  if (n_out <= 0) return cudaSuccess;
  minors_reduce_kernel<<<n_out, 32, 0, st>>>(plans, out_plans, out_begin, partials, out, nd_max);
  return cudaGetLastError();
}

}  // namespace boss
