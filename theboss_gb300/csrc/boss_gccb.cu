// boss_gccb.cu -- batched generalized Clifford & Clifford (version B) sampling.
//
// theboss draws one sample at a time (generalized_cliffords_b_simulation_strategy.py:41-110,
// generalized_cliffords_b_uniform_losses_simulation_strategy.py:87-121): per step it pops a
// random remaining input particle, computes the all-minors permanents of the
// current input against the output so far, expands them into the m output
// probabilities and draws one output mode.  Every random number it draws depends
// only on counts, never on a probability, so the host replays numpy's MT19937
// stream first (same calls, same order) and the GPU then runs all samples level
// by level:
//   level k (one graph node pair): the all-minors sweeps of every sample that has
//   >= k particles, as one launch of minors_sweep_kernel, then gccb_finalize_kernel
//   (one warp per sample): fixed-order reduction of the sweep partials, Laplace
//   expansion over the m outputs, |.|^2, normalisation with a sequential sum,
//   numpy.random.choice's cdf / searchsorted rule, and the sweep plan of the
//   sample's next level.
// The whole level loop is captured into one CUDA graph and launched once.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <numeric>
#include <vector>

#include "../../include/boss.h"
#include "boss_internal.h"

namespace boss {

extern std::mutex g_api_mutex;

// ---------------------------------------------------------------------------
// numpy legacy RandomState replay (MT19937, Matsumoto & Nishimura 1998).
// ---------------------------------------------------------------------------
struct MT19937 {
  uint32_t key[624];
  int pos;

  void twist() {
    const uint32_t upper = 0x80000000u, lower = 0x7fffffffu, a = 0x9908b0dfu;
    for (int i = 0; i < 624; ++i) {
      const uint32_t y = (key[i] & upper) | (key[(i + 1) % 624] & lower);
      key[i] = key[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? a : 0u);
    }
    pos = 0;
  }
  uint32_t next32() {
    if (pos >= 624) twist();
    uint32_t y = key[pos++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
  // 53-bit uniform in [0, 1): numpy.random.random / random_sample.
  double next_double() {
    const uint32_t a = next32() >> 5, b = next32() >> 6;
    return (a * 67108864.0 + b) / 9007199254740992.0;
  }
  // numpy.random.randint(0, n) for 1 <= n <= 2^32: masked rejection sampling on
  // 32-bit draws; n == 1 draws nothing.
  uint32_t bounded(uint64_t n) {
    const uint64_t rng = n - 1;
    if (rng == 0) return 0;
    uint32_t mask = (uint32_t)rng;
    mask |= mask >> 1;
    mask |= mask >> 2;
    mask |= mask >> 4;
    mask |= mask >> 8;
    mask |= mask >> 16;
    uint32_t v;
    while ((v = (next32() & mask)) > rng) {
    }
    return v;
  }
};

// The whole random stream of `n_samples` GC&C-B samples, in theboss's draw order.
static int predraw(const int32_t* input_state, int m, const double* weights, int n_weights, MT19937& mt,
                   int n_samples, std::vector<int32_t>& L, std::vector<uint8_t>& add, std::vector<double>& u,
                   int& n_particles) {
  std::vector<int> particles;
  for (int i = 0; i < m; ++i) {
    if (input_state[i] < 0 || input_state[i] > 255) {
      set_error("input occupations must be in [0, 255]");
      return kErrArg;
    }
    for (int k = 0; k < input_state[i]; ++k) particles.push_back(i);
  }
  const int n = (int)particles.size();
  n_particles = n;
  if (weights && n_weights != n + 1) {
    set_error("particle-number weights must have n + 1 entries");
    return kErrArg;
  }
  L.assign(n_samples, 0);
  add.assign((size_t)n_samples * std::max(n, 1), 0);
  u.assign((size_t)n_samples * std::max(n, 1), 0.0);
  std::vector<int> work;
  for (int s = 0; s < n_samples; ++s) {
    int l = n;
    if (weights) {  // generalized_cliffords_b_uniform_losses_simulation_strategy.py:67-85
      const double thr = mt.next_double();
      double acc = 0.0;
      l = 0;
      for (int i = 0; i < n_weights; ++i) {
        acc += weights[i];
        if (acc > thr) break;
        ++l;
      }
      if (l > n) {
        set_error("randint: low >= high (particle-number weights sum below the threshold)");
        return kErrArg;
      }
    }
    L[s] = l;
    work.assign(particles.begin(), particles.end());
    for (int k = 0; k < l; ++k) {  // generalized_cliffords_b_simulation_strategy.py:97-110
      const uint32_t idx = mt.bounded(work.size());
      add[(size_t)s * n + k] = (uint8_t)work[idx];
      work.erase(work.begin() + idx);
      u[(size_t)s * n + k] = mt.next_double();
    }
  }
  return kOk;
}

// ---------------------------------------------------------------------------
// Device side
// ---------------------------------------------------------------------------
struct LevelSample {  // host-computed layout of one sample's sweep at one level
  int64_t item_off;
  int64_t part_off;
  int64_t n_chunks;
  int64_t pool_off;
  int32_t n_items;
  int32_t c;
};

struct FinalizeArgs {
  int k;                 // level (number of input particles of this step)
  int A;                 // active samples at this level
  int A_next;            // active samples at level k + 1
  int m;
  int n;                 // add/u row stride
  const double2* U;
  uint8_t* S;            // [sample][m] current input occupations
  uint8_t* T;            // [sample][m] output occupations
  const uint8_t* add;    // [sample][n] popped input modes
  const double* uni;     // [sample][n] uniforms
  const SweepPlan* plans_cur;
  const uint8_t* dmode_cur;  // [sample][32]
  const double2* partials;
  SweepPlan* plans_next;
  uint8_t* dmode_next;
  double2* pool_next;
  const LevelSample* next_tab;  // A_next entries
  int* err;
};

constexpr int kFinWarps = 4;

__global__ void __launch_bounds__(kFinWarps * 32) gccb_finalize_kernel(FinalizeArgs a) {
  __shared__ double2 sub_s[kFinWarps][32];
  __shared__ uint8_t dm_s[kFinWarps][32];
  __shared__ uint8_t mult_s[kFinWarps][32];
  __shared__ uint8_t cm_s[kFinWarps][32];
  __shared__ uint8_t pw_s[kFinWarps][32];
  __shared__ double pmf_s[kFinWarps][256];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int j = blockIdx.x * kFinWarps + w;
  if (j >= a.A) return;
  const int m = a.m;
  uint8_t* S = a.S + (size_t)j * m;
  uint8_t* T = a.T + (size_t)j * m;
  int nd;
  if (a.k == 1) {
    // one particle: the minors are the input occupations themselves
    // (bs_submatrices_permanent_calculator_base.py:157-158)
    const int mode = a.add[(size_t)j * a.n];
    if (lane == 0) {
      S[mode] = 1;
      sub_s[w][0] = make_double2(1.0, 0.0);
      dm_s[w][0] = (uint8_t)mode;
      mult_s[w][0] = 1;
    }
    nd = 1;
  } else {
    const SweepPlan& P = a.plans_cur[j];
    nd = P.nd;
    if (lane < nd) {
      double sx = 0.0, sy = 0.0;
      for (int it = 0; it < P.n_items; ++it) {
        const double2 v = a.partials[P.part_off + (int64_t)it * nd + lane];
        sx += v.x;
        sy += v.y;
      }
      sub_s[w][lane] = make_double2(sx * P.scale, sy * P.scale);
      dm_s[w][lane] = a.dmode_cur[(size_t)j * 32 + lane];
      mult_s[w][lane] = P.mult[lane];
    }
  }
  __syncwarp();
  // Laplace expansion: perm(T + e_o) = sum_i S_i sub_i U[o][i]
  // (generalized_cliffords_b_simulation_strategy.py:82-89), then |.|^2.
  for (int o = lane; o < m; o += 32) {
    double re = 0.0, im = 0.0;
    for (int d = 0; d < nd; ++d) {
      const double2 s = sub_s[w][d];
      const double mu = (double)mult_s[w][d];
      const double2 u = a.U[(size_t)o * m + dm_s[w][d]];
      const double cr = mu * s.x, ci = mu * s.y;
      re = fma(cr, u.x, fma(-ci, u.y, re));
      im = fma(cr, u.y, fma(ci, u.x, im));
    }
    pmf_s[w][o] = fma(re, re, im * im);
  }
  __syncwarp();
  // Normalise with a sequential sum (Python's sum over the list), then
  // numpy.random.choice: cdf = cumsum(p); cdf /= cdf[-1]; searchsorted(cdf, u, 'right').
  double total = 0.0;
  if (lane == 0)
    for (int o = 0; o < m; ++o) total += pmf_s[w][o];
  total = __shfl_sync(0xffffffffu, total, 0);
  int idx = 0;
  if (!(total > 0.0) || !isfinite(total)) {
    if (lane == 0) atomicOr(a.err, 1);
  } else {
    for (int o = lane; o < m; o += 32) pmf_s[w][o] = pmf_s[w][o] / total;
    __syncwarp();
    if (lane == 0) {
      double c = 0.0;
      for (int o = 0; o < m; ++o) {
        c += pmf_s[w][o];
        pmf_s[w][o] = c;
      }
    }
    __syncwarp();
    const double last = pmf_s[w][m - 1];
    const double uu = a.uni[(size_t)j * a.n + (a.k - 1)];
    int cnt = 0;
    for (int o = lane; o < m; o += 32) cnt += (pmf_s[w][o] / last <= uu) ? 1 : 0;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, off);
    idx = cnt < m ? cnt : m - 1;
  }
  if (lane == 0) T[idx] = (uint8_t)(T[idx] + 1);
  __syncwarp();
  if (j >= a.A_next) return;

  // ---- plan of level k + 1 ----
  if (lane == 0) {
    const int mode = a.add[(size_t)j * a.n + a.k];
    S[mode] = (uint8_t)(S[mode] + 1);
  }
  __syncwarp();
  int nb = 0, nmul = 0, nc = 0, tsum = 0, all1 = 1;
  for (int base = 0; base < m; base += 32) {
    const int mode = base + lane;
    const int s = (mode < m) ? S[mode] : 0;
    const unsigned b1 = __ballot_sync(0xffffffffu, s == 1);
    if (s == 1) {
      const int pos = nb + __popc(b1 & ((1u << lane) - 1u));
      dm_s[w][pos] = (uint8_t)mode;
      mult_s[w][pos] = 1;
    }
    nb += __popc(b1);
  }
  for (int base = 0; base < m; base += 32) {
    const int mode = base + lane;
    const int s = (mode < m) ? S[mode] : 0;
    const unsigned bm = __ballot_sync(0xffffffffu, s > 1);
    if (s > 1) {
      const int pos = nb + nmul + __popc(bm & ((1u << lane) - 1u));
      dm_s[w][pos] = (uint8_t)mode;
      mult_s[w][pos] = (uint8_t)s;
    }
    nmul += __popc(bm);
  }
  for (int base = 0; base < m; base += 32) {
    const int mode = base + lane;
    const int t = (mode < m) ? T[mode] : 0;
    const unsigned bt = __ballot_sync(0xffffffffu, t > 0);
    if (t > 0) {
      const int pos = nc + __popc(bt & ((1u << lane) - 1u));
      cm_s[w][pos] = (uint8_t)mode;
      pw_s[w][pos] = (uint8_t)t;
    }
    nc += __popc(bt);
    tsum += __reduce_add_sync(0xffffffffu, (unsigned)t);
    all1 &= __all_sync(0xffffffffu, t <= 1);
  }
  __syncwarp();
  nd = nb + nmul;
  const LevelSample& ls = a.next_tab[j];
  double2* D = a.pool_next + ls.pool_off;
  for (int e = lane; e < nd * nc; e += 32) {
    const int d = e / nc, l = e - d * nc;
    D[e] = a.U[(size_t)cm_s[w][l] * m + dm_s[w][d]];
  }
  SweepPlan& P = a.plans_next[j];
  if (lane < 32) {
    P.mult[lane] = (lane < nd) ? mult_s[w][lane] : 0;
    P.mult[lane + 32] = 0;
    P.pw[lane] = (lane < nc) ? pw_s[w][lane] : 0;
    a.dmode_next[(size_t)j * 32 + lane] = (lane < nd) ? dm_s[w][lane] : 0;
  }
  if (lane == 0) {
    P.nd = nd;
    P.nb = nb;
    P.c = ls.c;
    P.nc = nc;
    P.kind = kRyser;
    P.parity0 = tsum & 1;  // multiplier (-1)^sum(T), bs_submatrices_permanent_calculator_base.py:185
    P.has_base = 0;
    P.all_pow1 = all1;
    P.n_chunks = ls.n_chunks;
    P.item_off = ls.item_off;
    P.n_items = ls.n_items;
    P.mat_off = ls.pool_off;
    P.base_off = 0;
    P.part_off = ls.part_off;
    P.code_off = 0;
    P.out_idx = j;
    P.reserved = 0;
    P.scale = 1.0;
  }
}

// ---------------------------------------------------------------------------
// Host orchestration
// ---------------------------------------------------------------------------
struct GccbGraphCache {
  cudaGraphExec_t exec = nullptr;
};
static GccbGraphCache g_graph;

static int run_gccb(Context* cx, const double* matrix, int m, int n, int N, const std::vector<int32_t>& L,
                    const std::vector<uint8_t>& add, const std::vector<double>& uni, int32_t* samples_out) {
  if (N == 0) return kOk;
  std::vector<int> order(N);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return L[x] > L[y]; });
  const int Lmax = L[order[0]];
  std::vector<int> A(Lmax + 2, 0);
  for (int s = 0; s < N; ++s)
    for (int k = 1; k <= L[s]; ++k) A[k]++;
  // Per-level layout (levels 2..Lmax need sweeps).
  const int64_t resident_warps = (int64_t)cx->sm_count * 12;
  std::vector<std::vector<LevelSample>> tab(Lmax + 2);
  std::vector<int64_t> lvl_items(Lmax + 2, 0), lvl_parts(Lmax + 2, 0), lvl_pool(Lmax + 2, 0);
  std::vector<int> lvl_c(Lmax + 2, 0);
  std::vector<uint8_t> occ(m);
  for (int k = 2; k <= Lmax; ++k) {
    const int Ak = A[k];
    std::vector<uint64_t> codes(Ak);
    std::vector<int> ndv(Ak), nbv(Ak);
    uint64_t total = 0;
    int min_nb = 64;
    for (int jj = 0; jj < Ak; ++jj) {
      const int s = order[jj];
      std::fill(occ.begin(), occ.end(), 0);
      for (int q = 0; q < k; ++q) occ[add[(size_t)s * n + q]]++;
      uint64_t c = 1;
      int nd = 0, nb = 0;
      for (int i = 0; i < m; ++i)
        if (occ[i]) {
          ++nd;
          if (occ[i] == 1) ++nb;
          c *= (uint64_t)occ[i] + 1;
        }
      codes[jj] = c;
      ndv[jj] = nd;
      nbv[jj] = nb;
      total += c;
      min_nb = std::min(min_nb, nb);
    }
    int c = 0;
    {
      const uint64_t per = total / (uint64_t)(32 * 8 * resident_warps);
      while (c < 12 && (1ull << (c + 1)) <= per) ++c;
      c = std::min(c, min_nb);
    }
    lvl_c[k] = c;
    auto& t = tab[k];
    t.resize(Ak);
    int64_t items = 0, parts = 0, pool = 0;
    for (int jj = 0; jj < Ak; ++jj) {
      LevelSample ls;
      ls.c = c;
      ls.n_chunks = (int64_t)(codes[jj] >> c);
      ls.n_items = (int32_t)((ls.n_chunks + 31) / 32);
      ls.item_off = items;
      ls.part_off = parts;
      ls.pool_off = pool;
      items += ls.n_items;
      parts += (int64_t)ls.n_items * ndv[jj];
      pool += (int64_t)ndv[jj] * (k - 1);
      t[jj] = ls;
    }
    lvl_items[k] = items;
    lvl_parts[k] = parts;
    lvl_pool[k] = pool;
  }
  int64_t max_parts = 1, max_pool = 1;
  for (int k = 2; k <= Lmax; ++k) {
    max_parts = std::max(max_parts, lvl_parts[k]);
    max_pool = std::max(max_pool, lvl_pool[k]);
  }
  // Arena (one H2D copy): counters | err | level tables | add | uniforms | U
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  size_t off = 0;
  const size_t o_cnt = off; off = al(off + sizeof(unsigned long long) * (Lmax + 2));
  const size_t o_err = off; off = al(off + sizeof(int));
  std::vector<size_t> o_tab(Lmax + 2, 0);
  for (int k = 2; k <= Lmax; ++k) { o_tab[k] = off; off = al(off + sizeof(LevelSample) * tab[k].size()); }
  const size_t o_add = off; off = al(off + (size_t)N * n);
  const size_t o_uni = off; off = al(off + sizeof(double) * (size_t)N * n);
  const size_t o_U = off; off = al(off + sizeof(double2) * (size_t)m * m);
  const size_t arena = off;
  int st;
  if ((st = ensure(cx->gccb[0], arena))) return st;
  if ((st = ensure(cx->gccb[1], (size_t)N * m * 2))) return st;                       // S | T
  if ((st = ensure(cx->gccb[2], sizeof(SweepPlan) * (size_t)A[1] * 2 + 512))) return st;  // plans x2
  if ((st = ensure(cx->gccb[3], (size_t)A[1] * 32 * 2))) return st;                   // dmode x2
  if ((st = ensure(cx->gccb[4], sizeof(double2) * (size_t)max_pool * 2 + 512))) return st;  // pool x2
  if ((st = ensure(cx->gccb[5], sizeof(double2) * (size_t)max_parts))) return st;    // partials
  if ((st = ensure_pinned(cx, std::max(arena, (size_t)N * m)))) return st;
  char* h = (char*)cx->pinned;
  memset(h, 0, o_add);
  for (int k = 2; k <= Lmax; ++k) memcpy(h + o_tab[k], tab[k].data(), sizeof(LevelSample) * tab[k].size());
  uint8_t* hadd = (uint8_t*)(h + o_add);
  double* huni = (double*)(h + o_uni);
  for (int jj = 0; jj < N; ++jj) {
    memcpy(hadd + (size_t)jj * n, &add[(size_t)order[jj] * n], n);
    memcpy(huni + (size_t)jj * n, &uni[(size_t)order[jj] * n], sizeof(double) * n);
  }
  memcpy(h + o_U, matrix, sizeof(double2) * (size_t)m * m);
  char* d = (char*)cx->gccb[0].ptr;
  uint8_t* dS = (uint8_t*)cx->gccb[1].ptr;
  uint8_t* dT = dS + (size_t)N * m;
  SweepPlan* plans[2] = {(SweepPlan*)cx->gccb[2].ptr, (SweepPlan*)cx->gccb[2].ptr + A[1]};
  uint8_t* dmode[2] = {(uint8_t*)cx->gccb[3].ptr, (uint8_t*)cx->gccb[3].ptr + (size_t)A[1] * 32};
  double2* pool[2] = {(double2*)cx->gccb[4].ptr, (double2*)cx->gccb[4].ptr + max_pool};
  double2* partials = (double2*)cx->gccb[5].ptr;
  cudaStream_t s = cx->stream;
  cudaError_t e = cudaMemcpyAsync(d, h, arena, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D sampler arena");

  // Capture the level loop into one graph.
  cudaGraph_t graph = nullptr;
  e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return fail_cuda(e, "begin capture");
  cudaError_t le = cudaMemsetAsync(dS, 0, (size_t)N * m * 2, s);
  for (int k = 1; k <= Lmax && le == cudaSuccess; ++k) {
    const int cur = k & 1, nxt = (k + 1) & 1;
    if (k >= 2) {
      SweepLaunch SL;
      SL.plans = plans[cur];
      SL.n_plans = A[k];
      SL.pool = pool[cur];
      SL.total_items = lvl_items[k];
      SL.counter = (unsigned long long*)(d + o_cnt) + k;
      SL.partials = partials;
      SL.max_nc = k - 1;
      SL.grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)cx->sm_count * 8, (lvl_items[k] + 3) / 4));
      le = launch_minors_sweep(SL, s);
      if (le != cudaSuccess) break;
    }
    FinalizeArgs fa;
    fa.k = k;
    fa.A = A[k];
    fa.A_next = (k < Lmax) ? A[k + 1] : 0;
    fa.m = m;
    fa.n = n;
    fa.U = (const double2*)(d + o_U);
    fa.S = dS;
    fa.T = dT;
    fa.add = (const uint8_t*)(d + o_add);
    fa.uni = (const double*)(d + o_uni);
    fa.plans_cur = plans[cur];
    fa.dmode_cur = dmode[cur];
    fa.partials = partials;
    fa.plans_next = plans[nxt];
    fa.dmode_next = dmode[nxt];
    fa.pool_next = pool[nxt];
    fa.next_tab = (k < Lmax) ? (const LevelSample*)(d + o_tab[k + 1]) : nullptr;
    fa.err = (int*)(d + o_err);
    gccb_finalize_kernel<<<(A[k] + kFinWarps - 1) / kFinWarps, kFinWarps * 32, 0, s>>>(fa);
    le = cudaGetLastError();
  }
  e = cudaStreamEndCapture(s, &graph);
  if (le != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    return fail_cuda(le, "sampler launch during capture");
  }
  if (e != cudaSuccess) return fail_cuda(e, "end capture");
  bool updated = false;
  if (g_graph.exec) {
    cudaGraphExecUpdateResultInfo info;
    if (cudaGraphExecUpdate(g_graph.exec, graph, &info) == cudaSuccess) updated = true;
    else {
      cudaGetLastError();
      cudaGraphExecDestroy(g_graph.exec);
      g_graph.exec = nullptr;
    }
  }
  if (!updated) {
    e = cudaGraphInstantiate(&g_graph.exec, graph, 0);
    if (e != cudaSuccess) {
      cudaGraphDestroy(graph);
      g_graph.exec = nullptr;
      return fail_cuda(e, "graph instantiate");
    }
  }
  cudaGraphDestroy(graph);
  e = cudaGraphLaunch(g_graph.exec, s);
  if (e != cudaSuccess) return fail_cuda(e, "graph launch");
  e = cudaMemcpyAsync(h, dT, (size_t)N * m, cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return fail_cuda(e, "D2H samples");
  int herr = 0;
  e = cudaMemcpyAsync(&herr, d + o_err, sizeof(int), cudaMemcpyDeviceToHost, s);
  if (e != cudaSuccess) return fail_cuda(e, "D2H status");
  e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail_cuda(e, "sampler");
  if (herr) {
    set_error("probabilities contain NaN (a pmf summed to zero or a non-finite value)");
    return kErrPmf;
  }
  const uint8_t* hT = (const uint8_t*)h;
  for (int jj = 0; jj < N; ++jj) {
    int32_t* row = samples_out + (size_t)order[jj] * m;
    for (int i = 0; i < m; ++i) row[i] = hT[(size_t)jj * m + i];
  }
  return kOk;
}

}  // namespace boss

using namespace boss;

static int load_mt(MT19937& mt, const uint32_t* key, const int32_t* pos) {
  if (!key || !pos || *pos < 0 || *pos > 624) {
    set_error("invalid MT19937 state");
    return kErrArg;
  }
  memcpy(mt.key, key, sizeof(mt.key));
  mt.pos = *pos;
  return kOk;
}

extern "C" {

int boss_gccb_predraw(const int32_t* input_state, int32_t m, const double* particle_weights, int32_t n_weights,
                      uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t* particles_kept,
                      int32_t* popped_modes, double* uniforms) {
  if (!input_state || m <= 0 || n_samples < 0 || !particles_kept) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  std::vector<int32_t> L;
  std::vector<uint8_t> add;
  std::vector<double> u;
  int n = 0;
  st = predraw(input_state, m, particle_weights, particle_weights ? n_weights : 0, mt, n_samples, L, add, u, n);
  if (st) return st;
  for (int s = 0; s < n_samples; ++s) {
    particles_kept[s] = L[s];
    for (int k = 0; k < n; ++k) {
      if (popped_modes) popped_modes[(size_t)s * n + k] = (k < L[s]) ? add[(size_t)s * n + k] : -1;
      if (uniforms) uniforms[(size_t)s * n + k] = (k < L[s]) ? u[(size_t)s * n + k] : 0.0;
    }
  }
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

int boss_gccb_sample(const double* matrix, int32_t m, const int32_t* input_state, const double* particle_weights,
                     int32_t n_weights, uint32_t* mt_key, int32_t* mt_pos, int32_t n_samples, int32_t* samples) {
  if (!matrix || !input_state || !samples || m <= 0 || n_samples < 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (m > 256) {
    set_error("the batched sampler supports at most 256 modes");
    return kErrLimit;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  MT19937 mt;
  int st = load_mt(mt, mt_key, mt_pos);
  if (st) return st;
  std::vector<int32_t> L;
  std::vector<uint8_t> add;
  std::vector<double> u;
  int n = 0;
  st = predraw(input_state, m, particle_weights, particle_weights ? n_weights : 0, mt, n_samples, L, add, u, n);
  if (st) return st;
  if (n > kMaxMinorDigits) {
    set_error("the batched sampler supports at most 32 input particles");
    return kErrLimit;
  }
  memset(samples, 0, sizeof(int32_t) * (size_t)n_samples * m);
  const bool any = std::any_of(L.begin(), L.end(), [](int32_t l) { return l > 0; });
  if (any) {
    Context* cx = context(&st);
    if (!cx) return st;
    st = run_gccb(cx, matrix, m, std::max(n, 1), n_samples, L, add, u, samples);
    if (st) return st;
  }
  memcpy(mt_key, mt.key, sizeof(mt.key));
  *mt_pos = mt.pos;
  return kOk;
}

}  // extern "C"
