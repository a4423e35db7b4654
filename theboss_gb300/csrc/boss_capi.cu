// boss_capi.cu -- host side of libboss_gb300.so: the per-process device context,
// the sweep planner (theboss calculator semantics -> SweepPlan segments) and the
// extern "C" entry points declared in include/boss.h.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/boss.h"
#include "boss_internal.h"

namespace boss {

static thread_local std::string g_last_error;
std::mutex g_api_mutex;

void set_error(const std::string& msg) { g_last_error = msg; }

int fail_cuda(cudaError_t e, const char* where) {
  set_error(std::string(where) + ": " + cudaGetErrorString(e));
  return kErrCuda;
}

static Context g_ctx;

Context* context(int* status) {
  *status = kOk;
  if (g_ctx.ready) return &g_ctx;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    set_error("no CUDA device available");
    *status = kErrNoDevice;
    return nullptr;
  }
  if ((e = cudaGetDevice(&g_ctx.device)) != cudaSuccess) { *status = fail_cuda(e, "cudaGetDevice"); return nullptr; }
  if ((e = cudaDeviceGetAttribute(&g_ctx.sm_count, cudaDevAttrMultiProcessorCount, g_ctx.device)) != cudaSuccess) {
    *status = fail_cuda(e, "cudaDeviceGetAttribute");
    return nullptr;
  }
  if ((e = cudaStreamCreateWithFlags(&g_ctx.stream, cudaStreamNonBlocking)) != cudaSuccess) {
    *status = fail_cuda(e, "cudaStreamCreate");
    return nullptr;
  }
  if ((e = prepare_sweep_kernels()) != cudaSuccess) {
    *status = fail_cuda(e, "kernel attributes");
    return nullptr;
  }
  g_ctx.ready = true;
  return &g_ctx;
}

int ensure(DeviceBuffer& b, size_t bytes) {
  if (bytes <= b.bytes && b.ptr) return kOk;
  size_t want = std::max(bytes, b.bytes + b.bytes / 2);
  want = (want + 4095) & ~(size_t)4095;
  if (b.ptr) cudaFree(b.ptr);
  b.ptr = nullptr;
  b.bytes = 0;
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMalloc");
  b.bytes = want;
  return kOk;
}

int ensure_pinned(Context* cx, size_t bytes) {
  if (bytes <= cx->pinned_bytes && cx->pinned) return kOk;
  size_t want = std::max(bytes, cx->pinned_bytes + cx->pinned_bytes / 2);
  want = (want + 4095) & ~(size_t)4095;
  if (cx->pinned) cudaFreeHost(cx->pinned);
  cx->pinned = nullptr;
  cx->pinned_bytes = 0;
  cudaError_t e = cudaMallocHost(&cx->pinned, want);
  if (e != cudaSuccess) return fail_cuda(e, "cudaMallocHost");
  cx->pinned_bytes = want;
  return kOk;
}

static inline size_t align_up(size_t x, size_t a) { return (x + a - 1) & ~(a - 1); }

static int ilog2_floor(uint64_t x) { return x ? 63 - __builtin_clzll(x) : 0; }

// Cuts sweeps into segments, uploads plans + matrices in one copy, launches the
// sweep and the reduction, and copies the results back.
int run_sweeps(Context* cx, const std::vector<HostSweep>& sweeps, bool minors, int nd_max, double2* results_host) {
  const int n_out = (int)sweeps.size();
  if (n_out == 0) return kOk;
  const int chunk_cap = minors ? 12 : 16;
  uint64_t total_all = 0;
  for (const auto& s : sweeps) total_all += s.total_codes;
  const uint64_t resident_warps = (uint64_t)cx->sm_count * 12;
  const int c_global = ilog2_floor(std::max<uint64_t>(1, total_all / (32ull * resident_warps * 8ull)));

  // pool: D then base of each sweep
  std::vector<int64_t> mat_off(n_out), base_off(n_out);
  int64_t pool_n = 0;
  for (int o = 0; o < n_out; ++o) {
    mat_off[o] = pool_n;
    pool_n += (int64_t)sweeps[o].D.size();
    base_off[o] = pool_n;
    pool_n += (int64_t)sweeps[o].base.size();
  }
  std::vector<SweepPlan> big, small;
  int max_nc = 1;
  for (int o = 0; o < n_out; ++o) {
    const HostSweep& s = sweeps[o];
    max_nc = std::max(max_nc, s.nc);
    SweepPlan p;
    memset(&p, 0, sizeof(p));
    p.nd = s.nd;
    p.nb = s.nb;
    p.nc = s.nc;
    p.kind = s.kind;
    p.parity0 = s.parity0;
    p.has_base = s.has_base;
    p.all_pow1 = 1;
    for (int l = 0; l < s.nc; ++l) {
      p.pw[l] = s.pw[l];
      if (s.pw[l] != 1) p.all_pow1 = 0;
    }
    for (int i = 0; i < s.nd; ++i) p.mult[i] = s.mult[i];
    p.mat_off = mat_off[o];
    p.base_off = base_off[o];
    p.scale = s.scale;
    p.out_idx = o;
    const uint64_t T = s.total_codes;
    int c = std::min(std::min(c_global, s.nb), chunk_cap);
    c = std::min(c, ilog2_floor(std::max<uint64_t>(1, T / 32)));
    c = std::max(c, 0);
    const uint64_t nch = T >> c;
    if (nch >= 256 && c >= 3) {
      const uint64_t a = nch - nch / 8;
      SweepPlan p1 = p;
      p1.c = c;
      p1.code_off = 0;
      p1.n_chunks = (int64_t)a;
      big.push_back(p1);
      SweepPlan p2 = p;
      p2.c = c - 3;
      p2.code_off = (int64_t)(a << c);
      p2.n_chunks = (int64_t)((T - (a << c)) >> (c - 3));
      small.push_back(p2);
    } else {
      SweepPlan p1 = p;
      p1.c = c;
      p1.code_off = 0;
      p1.n_chunks = (int64_t)nch;
      big.push_back(p1);
    }
  }
  std::vector<SweepPlan> plans(big);
  plans.insert(plans.end(), small.begin(), small.end());
  const int n_plans = (int)plans.size();
  int64_t items = 0, parts = 0;
  for (auto& p : plans) {
    p.n_items = (p.n_chunks + 31) / 32;
    p.item_off = items;
    p.part_off = parts;
    items += p.n_items;
    parts += p.n_items * (minors ? p.nd : 1);
  }
  std::vector<int32_t> out_plans(n_plans), out_begin(n_out + 1, 0);
  for (int i = 0; i < n_plans; ++i) out_begin[plans[i].out_idx + 1]++;
  for (int o = 0; o < n_out; ++o) out_begin[o + 1] += out_begin[o];
  {
    std::vector<int32_t> fill(out_begin.begin(), out_begin.end() - 1);
    for (int i = 0; i < n_plans; ++i) out_plans[fill[plans[i].out_idx]++] = i;
  }

  // arena: counter | plans | out_plans | out_begin | pool
  size_t off = 0;
  const size_t o_counter = off; off = align_up(off + 16, 256);
  const size_t o_plans = off; off = align_up(off + sizeof(SweepPlan) * n_plans, 256);
  const size_t o_oplans = off; off = align_up(off + sizeof(int32_t) * n_plans, 256);
  const size_t o_obegin = off; off = align_up(off + sizeof(int32_t) * (n_out + 1), 256);
  const size_t o_pool = off; off = align_up(off + sizeof(double2) * std::max<int64_t>(pool_n, 1), 256);
  const size_t arena_bytes = off;
  const size_t out_elems = (size_t)n_out * (minors ? nd_max : 1);
  int st;
  if ((st = ensure(cx->plans, arena_bytes))) return st;
  if ((st = ensure(cx->partials, sizeof(double2) * std::max<int64_t>(parts, 1)))) return st;
  if ((st = ensure(cx->out, sizeof(double2) * out_elems))) return st;
  if ((st = ensure_pinned(cx, std::max(arena_bytes, sizeof(double2) * out_elems)))) return st;
  char* h = (char*)cx->pinned;
  memset(h + o_counter, 0, 16);
  memcpy(h + o_plans, plans.data(), sizeof(SweepPlan) * n_plans);
  memcpy(h + o_oplans, out_plans.data(), sizeof(int32_t) * n_plans);
  memcpy(h + o_obegin, out_begin.data(), sizeof(int32_t) * (n_out + 1));
  double2* hp = (double2*)(h + o_pool);
  for (int o = 0; o < n_out; ++o) {
    std::copy(sweeps[o].D.begin(), sweeps[o].D.end(), hp + mat_off[o]);
    std::copy(sweeps[o].base.begin(), sweeps[o].base.end(), hp + base_off[o]);
  }
  char* d = (char*)cx->plans.ptr;
  cudaError_t e = cudaMemcpyAsync(d, h, arena_bytes, cudaMemcpyHostToDevice, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "H2D plans");
  SweepLaunch L;
  L.plans = (const SweepPlan*)(d + o_plans);
  L.n_plans = n_plans;
  L.pool = (const double2*)(d + o_pool);
  L.total_items = items;
  L.counter = (unsigned long long*)(d + o_counter);
  L.partials = (double2*)cx->partials.ptr;
  L.max_nc = max_nc;
  L.grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)cx->sm_count * 8, (items + 3) / 4));
  e = minors ? launch_minors_sweep(L, cx->stream) : launch_perm_sweep(L, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "sweep launch");
  e = minors ? launch_minors_reduce(L.plans, (const int32_t*)(d + o_oplans), (const int32_t*)(d + o_obegin), n_out,
                                    L.partials, (double2*)cx->out.ptr, nd_max, cx->stream)
             : launch_perm_reduce(L.plans, (const int32_t*)(d + o_oplans), (const int32_t*)(d + o_obegin), n_out,
                                  L.partials, (double2*)cx->out.ptr, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "reduce launch");
  e = cudaMemcpyAsync(cx->pinned, cx->out.ptr, sizeof(double2) * out_elems, cudaMemcpyDeviceToHost, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "D2H results");
  e = cudaStreamSynchronize(cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "sweep");
  memcpy(results_host, cx->pinned, sizeof(double2) * out_elems);
  return kOk;
}

// ---------------------------------------------------------------------------
// Planner: theboss calculator semantics -> HostSweep
// ---------------------------------------------------------------------------
static inline double2 U_at(const double* U, int m, int row, int col) {
  const double* p = U + 2 * ((size_t)row * m + col);
  return make_double2(p[0], p[1]);
}

struct Side {
  int n = 0;                 // particles
  std::vector<int> modes;    // distinct occupied modes, binary first
  std::vector<int> mult;
  int nb = 0;
  uint64_t codes = 1;        // prod (mult + 1)
};

static Side make_side(const int32_t* occ, int len) {
  Side s;
  for (int i = 0; i < len; ++i)
    if (occ[i] == 1) { s.modes.push_back(i); s.mult.push_back(1); }
  s.nb = (int)s.modes.size();
  for (int i = 0; i < len; ++i)
    if (occ[i] > 1) { s.modes.push_back(i); s.mult.push_back(occ[i]); }
  for (int i = 0; i < len; ++i) s.n += std::max(occ[i], 0);
  for (size_t a = 0; a < s.mult.size(); ++a) {
    const uint64_t b = (uint64_t)s.mult[a] + 1;
    s.codes = (s.codes > (UINT64_MAX >> 2) / b) ? UINT64_MAX : s.codes * b;
  }
  return s;
}

// Fills a sweep that iterates `dig` and multiplies over `col`.  entry(a, l) gives
// the matrix element between digit mode a and column mode l.
template <class F>
static int fill_sweep(HostSweep& hs, const Side& dig, const Side& col, int kind, bool halve, F entry) {
  int drop = -1;
  if (halve && dig.nb > 0) drop = dig.nb - 1;  // a binary digit fixed at r = 0
  hs.kind = kind;
  hs.nd = (int)dig.modes.size() - (drop >= 0 ? 1 : 0);
  hs.nb = dig.nb - (drop >= 0 ? 1 : 0);
  hs.nc = (int)col.modes.size();
  if (hs.nd > kMaxDigits || hs.nc > kMaxCols) {
    set_error("sweep exceeds 64 distinct iterated modes or 32 distinct product modes");
    return kErrLimit;
  }
  hs.total_codes = 1;
  int a_out = 0;
  for (size_t a = 0; a < dig.modes.size(); ++a) {
    if ((int)a == drop) continue;
    hs.mult[a_out] = (uint8_t)dig.mult[a];
    hs.digit_mode[a_out] = dig.modes[a];
    const uint64_t b = (uint64_t)dig.mult[a] + 1;
    if (hs.total_codes > (1ull << 62) / b) {
      set_error("code count exceeds 2^62");
      return kErrLimit;
    }
    hs.total_codes *= b;
    ++a_out;
  }
  for (int l = 0; l < hs.nc; ++l) hs.pw[l] = (uint8_t)col.mult[l];
  hs.D.resize((size_t)hs.nd * hs.nc);
  const double f = (kind == kGlynn) ? 2.0 : 1.0;
  a_out = 0;
  for (size_t a = 0; a < dig.modes.size(); ++a) {
    if ((int)a == drop) continue;
    for (int l = 0; l < hs.nc; ++l) {
      const double2 z = entry(dig.modes[a], col.modes[l]);
      hs.D[(size_t)a_out * hs.nc + l] = make_double2(f * z.x, f * z.y);
    }
    ++a_out;
  }
  hs.has_base = (kind == kGlynn);
  if (hs.has_base) {
    hs.base.assign(hs.nc, make_double2(0.0, 0.0));
    for (int l = 0; l < hs.nc; ++l) {
      double re = 0.0, im = 0.0;
      for (size_t a = 0; a < dig.modes.size(); ++a) {
        const double2 z = entry(dig.modes[a], col.modes[l]);
        re += dig.mult[a] * z.x;
        im += dig.mult[a] * z.y;
      }
      hs.base[l] = make_double2(re, im);
    }
    hs.scale = std::ldexp(1.0, -dig.n) * (drop >= 0 ? 2.0 : 1.0);
    hs.parity0 = 0;
  } else {
    hs.scale = 1.0;
    hs.parity0 = dig.n & 1;
  }
  return kOk;
}

// One permanent request.  Returns kOk and either fills `hs` (needs_sweep = true)
// or sets `value` directly for the edge cases theboss special-cases.
static int plan_permanent(const double* U, int m, const int32_t* S, const int32_t* T, int len, int variant,
                          HostSweep& hs, bool& needs_sweep, double2& value) {
  needs_sweep = false;
  if (len > m || len < 0) {  // bs_permanent_calculator_base.py:61-72
    set_error("state length exceeds matrix dimension");
    return kErrSize;
  }
  for (int i = 0; i < len; ++i)
    if (S[i] < 0 || T[i] < 0 || S[i] > 255 || T[i] > 255) {
      set_error("occupations must be in [0, 255]");
      return kErrArg;
    }
  const Side in = make_side(S, len), out = make_side(T, len);
  auto entry_in_out = [&](int i_mode, int j_mode) { return U_at(U, m, j_mode, i_mode); };  // digit = input
  auto entry_out_in = [&](int j_mode, int i_mode) { return U_at(U, m, j_mode, i_mode); };  // digit = output
  switch (variant) {
    case BOSS_RYSER:
    case BOSS_CHIN_HUH: {
      if (out.modes.empty()) {  // empty product: (1 - 1)^n
        value = make_double2(in.n == 0 ? 1.0 : 0.0, 0.0);
        return kOk;
      }
      if (in.modes.empty()) {  // r = 0 only: prod of zero sums
        value = make_double2(0.0, 0.0);
        return kOk;
      }
      const bool ch = (variant == BOSS_CHIN_HUH);
      const int st = fill_sweep(hs, in, out, ch ? kGlynn : kRyser, ch && in.n == out.n, entry_in_out);
      if (st) return st;
      needs_sweep = true;
      return kOk;
    }
    case BOSS_GLYNN:
    case BOSS_CLASSIC: {
      if (variant == BOSS_CLASSIC && in.n == 0) {  // classic_permanent_calculator.py:29-33
        value = make_double2(out.n == 0 ? 1.0 : 0.0, 0.0);
        return kOk;
      }
      if (in.n == 0 || out.n == 0) {  // glynn_gray_permanent_calculator.py:52-53
        value = make_double2(1.0, 0.0);
        return kOk;
      }
      if (in.n != out.n) {
        set_error("effective scattering matrix is not square (sum of input != sum of output)");
        return kErrSize;
      }
      // Iterate the side with fewer codes (after fixing one binary digit).
      const uint64_t ci = in.nb ? in.codes / 2 : in.codes;
      const uint64_t co = out.nb ? out.codes / 2 : out.codes;
      int st;
      if (co < ci || (co == ci && out.modes.size() <= kMaxDigits && in.modes.size() > kMaxCols))
        st = fill_sweep(hs, out, in, kGlynn, true, entry_out_in);
      else
        st = fill_sweep(hs, in, out, kGlynn, true, entry_in_out);
      if (st == kErrLimit) {  // try the other orientation
        if (co < ci) st = fill_sweep(hs, in, out, kGlynn, true, entry_in_out);
        else st = fill_sweep(hs, out, in, kGlynn, true, entry_out_in);
      }
      if (st) return st;
      if (hs.nd == 0) {  // a single code
        // fall through to the sweep anyway: nd = 0 is a one-code sweep
      }
      needs_sweep = true;
      return kOk;
    }
    default:
      set_error("unknown permanent variant");
      return kErrArg;
  }
}

// All-minors request (bs_submatrices_permanent_calculator_base.py:150-189).
// results: len complex (minor of input mode i at position i).
static int plan_minors(const double* U, int m, const int32_t* S, const int32_t* T, int len, HostSweep& hs,
                       bool& needs_sweep, double2* direct) {
  needs_sweep = false;
  if (len > m || len <= 0) {
    set_error("state length must be in [1, matrix dimension]");
    return kErrSize;
  }
  for (int i = 0; i < len; ++i)
    if (S[i] < 0 || T[i] < 0 || S[i] > 255 || T[i] > 255) {
      set_error("occupations must be in [0, 255]");
      return kErrArg;
    }
  const Side in = make_side(S, len), out = make_side(T, len);
  if (in.n == 1) {  // bs_submatrices_permanent_calculator_base.py:157-158
    for (int i = 0; i < len; ++i) direct[i] = make_double2((double)S[i], 0.0);
    return kOk;
  }
  for (int i = 0; i < len; ++i) direct[i] = make_double2(0.0, 0.0);
  if (in.n == 0) return kOk;
  if (in.modes.size() > (size_t)kMaxMinorDigits || out.modes.size() > (size_t)kMaxCols) {
    set_error("all-minors sweep exceeds 32 distinct input or output modes");
    return kErrLimit;
  }
  if (out.modes.empty()) {
    // Product over no columns is 1; theboss skips the r = 0 code
    // (bs_cc_ryser_submatrices_permanent_calculator.py:73-78), so every other code
    // adds (-1)^|r| C-weights.  Evaluated directly on the host.
    std::vector<int> r(in.modes.size(), 0), u(in.modes.size(), 1);
    double binom = 1.0;
    double sign = 1.0;
    const size_t nd = in.modes.size();
    uint64_t guard = 0;
    for (;;) {
      size_t idx = 0;
      int k = r[0] + u[0];
      bool done = false;
      while (k > in.mult[idx] || k < 0) {
        u[idx] = -u[idx];
        if (++idx == nd) { done = true; break; }
        k = r[idx] + u[idx];
      }
      if (done) break;
      const int last = r[idx];
      r[idx] = k;
      sign = -sign;
      binom = (k > last) ? binom * ((double)(in.mult[idx] - last) / k) : binom * ((double)last / (in.mult[idx] - k));
      for (size_t a = 0; a < nd; ++a) {
        if (r[a] == in.mult[a]) continue;
        const double ub = binom / ((double)in.mult[a] / (in.mult[a] - r[a]));
        direct[in.modes[a]].x += sign * ub;
      }
      if (++guard > (1ull << 24)) {
        set_error("degenerate all-minors request too large");
        return kErrLimit;
      }
    }
    return kOk;
  }
  auto entry = [&](int i_mode, int j_mode) { return U_at(U, m, j_mode, i_mode); };
  const int st = fill_sweep(hs, in, out, kRyser, false, entry);
  if (st) return st;
  hs.parity0 = out.n & 1;  // multiplier (-1)^sum(T), bs_submatrices_permanent_calculator_base.py:185
  needs_sweep = true;
  return kOk;
}

}  // namespace boss

using namespace boss;

extern "C" {

const char* boss_last_error(void) { return g_last_error.c_str(); }

int boss_abi_version(void) { return BOSS_ABI_VERSION; }

int boss_device_sm_count(int32_t* sm_count) {
  std::lock_guard<std::mutex> lk(g_api_mutex);
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  *sm_count = cx->sm_count;
  return kOk;
}

int boss_perm_batch(const double* matrix, int32_t m, const int32_t* input_states, const int32_t* output_states,
                    int32_t len, int32_t count, int32_t variant, double* results) {
  if (!matrix || !input_states || !output_states || !results || m <= 0 || count < 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  std::vector<HostSweep> sweeps;
  std::vector<int> which;
  sweeps.reserve(count);
  for (int k = 0; k < count; ++k) {
    HostSweep hs;
    bool need = false;
    double2 v = make_double2(0.0, 0.0);
    const int st = plan_permanent(matrix, m, input_states + (size_t)k * len, output_states + (size_t)k * len, len,
                                  variant, hs, need, v);
    if (st) return st;
    if (need) {
      sweeps.push_back(std::move(hs));
      which.push_back(k);
    } else {
      results[2 * k] = v.x;
      results[2 * k + 1] = v.y;
    }
  }
  if (sweeps.empty()) return kOk;
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  std::vector<double2> out(sweeps.size());
  st = run_sweeps(cx, sweeps, false, 1, out.data());
  if (st) return st;
  for (size_t a = 0; a < which.size(); ++a) {
    results[2 * which[a]] = out[a].x;
    results[2 * which[a] + 1] = out[a].y;
  }
  return kOk;
}

int boss_submatrices_batch(const double* matrix, int32_t m, const int32_t* input_states,
                           const int32_t* output_states, int32_t len, int32_t count, int32_t variant,
                           double* results) {
  if (!matrix || !input_states || !output_states || !results || m <= 0 || count < 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  if (variant != BOSS_RYSER && variant != BOSS_CHIN_HUH) {
    set_error("all-minors variant must be BOSS_RYSER or BOSS_CHIN_HUH");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  std::vector<HostSweep> sweeps;
  std::vector<int> which;
  double2* res = (double2*)results;
  for (int k = 0; k < count; ++k) {
    HostSweep hs;
    bool need = false;
    const int st = plan_minors(matrix, m, input_states + (size_t)k * len, output_states + (size_t)k * len, len, hs,
                               need, res + (size_t)k * len);
    if (st) return st;
    if (need) {
      sweeps.push_back(std::move(hs));
      which.push_back(k);
    }
  }
  if (sweeps.empty()) return kOk;
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  const int nd_max = kMaxMinorDigits;
  std::vector<double2> out(sweeps.size() * nd_max);
  st = run_sweeps(cx, sweeps, true, nd_max, out.data());
  if (st) return st;
  for (size_t a = 0; a < which.size(); ++a) {
    const HostSweep& hs = sweeps[a];
    double2* row = res + (size_t)which[a] * len;
    for (int d = 0; d < hs.nd; ++d) row[hs.digit_mode[d]] = out[a * nd_max + d];
  }
  return kOk;
}

}  // extern "C"
