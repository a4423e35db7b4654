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
  for (cudaStream_t& st : g_ctx.sampler_streams)
    if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) {
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

// A list of sweeps that share one factor count, uploaded and ready to launch.
struct SweepBatch {
  int n = 0, nf = 0;
  bool minors = false;
  bool ff = false;  // all-minors on float pairs
  int nd_max = 1;
  SweepLaunch L;
  size_t out_elems = 0;
  double codes = 0.0;  // codes swept per launch
};

static int sweeps_prepare(Context* cx, const std::vector<HostSweep>& sweeps, bool minors, int nd_max, SweepBatch& B) {
  const int n = (int)sweeps.size();
  B.n = n;
  B.nf = sweeps[0].nf;
  B.minors = minors;
  B.nd_max = nd_max;
  // Float pairs only for Glynn-kind sweeps: the Ryser form's alternating sum cancels
  // far more (its FP64 error is already ~1e-10 at n = 20), and float pairs would
  // leave theboss's tolerance.
  bool glynn = true;
  for (const HostSweep& h : sweeps) glynn = glynn && h.kind == kGlynn;
  B.ff = glynn && (minors ? (g_minors_arith == 0 && minors_ff_available(B.nf))
                          : (g_perm_arith == 0 && perm_ff_available(B.nf)));
  const SweepOp op = minors ? SweepOp::kMinors : (B.ff ? SweepOp::kPermFF : SweepOp::kPerm);
  std::vector<uint64_t> codes(n);
  B.codes = 0.0;
  for (int p = 0; p < n; ++p) {
    codes[p] = sweeps[p].total_codes;
    B.codes += (double)codes[p];
  }
  int rows = 1;  // all-minors: shared-memory rows of minors per thread
  for (int p = 0; p < n; ++p) rows = std::max(rows, sweeps[p].nd + (sweeps[p].fixed_mode >= 0 ? 1 : 0));
  std::vector<int64_t> nthr;
  partition_threads(codes,
                    minors ? sweep_resident_minors(B.nf, rows, cx->sm_count, B.ff)
                           : sweep_resident_threads(B.nf, op, cx->sm_count),
                    nthr);
  std::vector<SweepProblem> probs(n);
  int64_t pool_n = 0, threads = 0, parts = 0;
  for (int p = 0; p < n; ++p) {
    const HostSweep& h = sweeps[p];
    SweepProblem& P = probs[p];
    memset(&P, 0, sizeof(P));
    P.nd = h.nd;
    P.nb = h.nb;
    P.nf = h.nf;
    P.kind = h.kind;
    P.parity0 = h.parity0;
    P.fx = h.fx;
    P.has_base = h.has_base;
    P.out_idx = p;
    P.n_codes = (int64_t)h.total_codes;
    P.thread_begin = threads;
    P.n_threads = nthr[p];
    P.mat_off = pool_n;
    pool_n += (int64_t)h.D.size();
    P.base_off = pool_n;
    pool_n += (int64_t)h.base.size();
    P.part_off = parts;
    P.scale = h.scale;
    if (B.ff) {  // float-pair rows of the binary digits, then the factors' biases
      P.ff_off = pool_n;
      pool_n += (int64_t)h.nb * h.nf + (h.nf + 3) / 4;
      P.scale = std::ldexp(h.scale, h.ff_exp);
    }
    P.fixed_digit = (h.fixed_mode >= 0) ? 1 : 0;
    for (int i = 0; i < h.nd; ++i) P.mult[i] = h.mult[i];
    threads += nthr[p];
    parts += nthr[p] * (minors ? h.nd + P.fixed_digit : 1);
  }
  // arena: problems | pool
  size_t off = 0;
  const size_t o_probs = off; off = align_up(off + sizeof(SweepProblem) * n, 256);
  const size_t o_pool = off; off = align_up(off + sizeof(longlong2) * std::max<int64_t>(pool_n, 1), 256);
  const size_t arena_bytes = off;
  B.out_elems = (size_t)n * (minors ? nd_max : 1);
  int st;
  if ((st = ensure(cx->plans, arena_bytes))) return st;
  if ((st = ensure(cx->partials, sizeof(double2) * std::max<int64_t>(parts, 1)))) return st;
  if ((st = ensure(cx->out, sizeof(double2) * B.out_elems))) return st;
  if ((st = ensure_pinned(cx, std::max(arena_bytes, sizeof(double2) * B.out_elems)))) return st;
  char* h = (char*)cx->pinned;
  memcpy(h + o_probs, probs.data(), sizeof(SweepProblem) * n);
  longlong2* hp = (longlong2*)(h + o_pool);
  for (int p = 0; p < n; ++p) {
    const HostSweep& hs = sweeps[p];
    std::copy(hs.D.begin(), hs.D.end(), hp + probs[p].mat_off);
    std::copy(hs.base.begin(), hs.base.end(), hp + probs[p].base_off);
    if (B.ff) {
      float4* df = reinterpret_cast<float4*>(hp + probs[p].ff_off);
      for (int d = 0; d < hs.nb; ++d)
        for (int f = 0; f < hs.nf; ++f) {
          const longlong2 v = hs.D[(size_t)d * hs.nf + f];
          float4& o = df[(size_t)d * hs.nf + f];
          host_fx_to_ff(v.x, hs.fbias[f], o.x, o.y);
          host_fx_to_ff(v.y, hs.fbias[f], o.z, o.w);
        }
      int* fb = reinterpret_cast<int*>(df + (size_t)hs.nb * hs.nf);
      for (int f = 0; f < hs.nf; ++f) fb[f] = hs.fbias[f];
    }
  }
  char* d = (char*)cx->plans.ptr;
  cudaError_t e = cudaMemcpyAsync(d, h, arena_bytes, cudaMemcpyHostToDevice, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "H2D sweeps");
  B.L.probs = (const SweepProblem*)(d + o_probs);
  B.L.n_probs = n;
  B.L.pool = (const longlong2*)(d + o_pool);
  B.L.total_threads = threads;
  B.L.partials = (double2*)cx->partials.ptr;
  B.L.grid = (int)((threads + 127) / 128);
  B.L.rows = rows;
  return kOk;
}

static int sweeps_launch(Context* cx, const SweepBatch& B, cudaEvent_t after_sweep = nullptr) {
  const SweepOp op = B.minors ? (B.ff ? SweepOp::kMinorsFF : SweepOp::kMinors) : (B.ff ? SweepOp::kPermFF : SweepOp::kPerm);
  cudaError_t e = launch_sweep(B.nf, op, B.L, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "sweep launch");
  if (after_sweep) cudaEventRecord(after_sweep, cx->stream);
  e = B.minors ? launch_minors_reduce(B.L.probs, B.n, B.L.partials, (double2*)cx->out.ptr, B.nd_max, cx->stream, B.ff)
               : launch_perm_reduce(B.L.probs, B.n, B.L.partials, (double2*)cx->out.ptr, cx->stream, B.ff);
  return e == cudaSuccess ? kOk : fail_cuda(e, "reduce launch");
}

static int sweeps_collect(Context* cx, const SweepBatch& B, double2* results_host) {
  cudaError_t e =
      cudaMemcpyAsync(cx->pinned, cx->out.ptr, sizeof(double2) * B.out_elems, cudaMemcpyDeviceToHost, cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "D2H results");
  e = cudaStreamSynchronize(cx->stream);
  if (e != cudaSuccess) return fail_cuda(e, "sweep");
  memcpy(results_host, cx->pinned, sizeof(double2) * B.out_elems);
  return kOk;
}

int run_sweeps(Context* cx, const std::vector<HostSweep>& sweeps, bool minors, int nd_max, double2* results_host) {
  if (sweeps.empty()) return kOk;
  SweepBatch B;
  int st = sweeps_prepare(cx, sweeps, minors, nd_max, B);
  if (st) return st;
  if ((st = sweeps_launch(cx, B))) return st;
  return sweeps_collect(cx, B, results_host);
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

// Fixed-point fraction bits for sums bounded by `bound` (|s| <= bound): the
// integer sums stay below 2^61.
static int choose_fx(double bound) {
  if (!(bound > 0.0) || !std::isfinite(bound)) return 56;
  int ex = 0;
  std::frexp(bound, &ex);  // bound < 2^ex
  int fx = 61 - ex;
  return std::max(-900, std::min(fx, 200));
}

static inline long long to_fixed(double v, int fx) { return std::llrint(std::ldexp(v, fx)); }

// Fills a sweep that iterates `dig` and multiplies over the particles of `col`
// (a mode occupied p times gives p factors).  entry(a, l) is the matrix element
// between digit mode a and product mode l.
template <class F>
static int fill_sweep(HostSweep& hs, const Side& dig, const Side& col, int kind, bool halve, F entry) {
  int drop = -1;
  if (halve && dig.nb > 0) drop = dig.nb - 1;  // a binary digit fixed at r = 0
  hs.kind = kind;
  hs.nd = (int)dig.modes.size() - (drop >= 0 ? 1 : 0);
  hs.nb = dig.nb - (drop >= 0 ? 1 : 0);
  std::vector<int> fmode;
  for (size_t l = 0; l < col.modes.size(); ++l)
    for (int k = 0; k < col.mult[l]; ++k) fmode.push_back(col.modes[l]);
  hs.nf = (int)fmode.size();
  hs.fixed_mode = (drop >= 0) ? dig.modes[drop] : -1;
  for (int f = 0; f < (int)fmode.size() && f < kMaxFactors; ++f) hs.factor_mode[f] = fmode[f];
  if (hs.nd > kMaxDigits || hs.nf > kMaxFactors || hs.nf < 1) {
    set_error("sweep exceeds 64 distinct iterated modes or 32 product-side particles");
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
  // |row sum| <= sum_a mult_a * max component of the entries
  double bound = 0.0;
  for (size_t a = 0; a < dig.modes.size(); ++a) {
    double mx = 0.0;
    for (int f = 0; f < hs.nf; ++f) {
      const double2 z = entry(dig.modes[a], fmode[f]);
      mx = std::max(mx, std::max(std::fabs(z.x), std::fabs(z.y)));
    }
    bound += dig.mult[a] * mx;
  }
  hs.fx = choose_fx(bound);
  hs.D.resize((size_t)hs.nd * hs.nf);
  const long long fsign = (kind == kGlynn) ? -2 : 1;  // Glynn: s = base - 2 sum r U
  a_out = 0;
  for (size_t a = 0; a < dig.modes.size(); ++a) {
    if ((int)a == drop) continue;
    for (int f = 0; f < hs.nf; ++f) {
      const double2 z = entry(dig.modes[a], fmode[f]);
      longlong2 v;
      v.x = fsign * to_fixed(z.x, hs.fx);
      v.y = fsign * to_fixed(z.y, hs.fx);
      hs.D[(size_t)a_out * hs.nf + f] = v;
    }
    ++a_out;
  }
  hs.has_base = (kind == kGlynn);
  if (hs.has_base) {
    hs.base.assign(hs.nf, longlong2{0, 0});
    for (int f = 0; f < hs.nf; ++f) {
      long long re = 0, im = 0;
      for (size_t a = 0; a < dig.modes.size(); ++a) {
        const double2 z = entry(dig.modes[a], fmode[f]);
        re += (long long)dig.mult[a] * to_fixed(z.x, hs.fx);
        im += (long long)dig.mult[a] * to_fixed(z.y, hs.fx);
      }
      hs.base[f].x = re;
      hs.base[f].y = im;
    }
    hs.scale = std::ldexp(1.0, -dig.n) * (drop >= 0 ? 2.0 : 1.0);
    hs.parity0 = 0;
  } else {
    hs.scale = 1.0;
    hs.parity0 = dig.n & 1;
  }
  hs.fbias.assign(hs.nf, 189);
  hs.ff_exp = 0;
  for (int f = 0; f < hs.nf; ++f) {
    unsigned long long bx = 0, by = 0;
    for (size_t a = 0; a < dig.modes.size(); ++a) {
      const double2 z = entry(dig.modes[a], fmode[f]);
      bx += (unsigned long long)dig.mult[a] * (unsigned long long)std::llabs(to_fixed(z.x, hs.fx));
      by += (unsigned long long)dig.mult[a] * (unsigned long long)std::llabs(to_fixed(z.y, hs.fx));
    }
    const unsigned long long b = std::max(bx, by);
    const int p = b ? 63 - __builtin_clzll(b) : 0;
    hs.fbias[f] = 189 - p;
    hs.ff_exp += p + 1 - hs.fx;
  }
  return kOk;
}

// FP64 by default (theboss computes in float64); float pairs on request.
int g_minors_arith = 1;
int g_perm_arith = 1;

void host_fx_to_ff(long long x, int fbias, float& hi, float& lo) {
  const unsigned long long sgn = (unsigned long long)(x >> 63);
  const unsigned long long ax = ((unsigned long long)x ^ sgn) - sgn;
  if (!ax) {
    hi = lo = 0.0f;
    return;
  }
  const int lz = __builtin_clzll(ax);
  const unsigned long long y = ax << lz;
  const uint32_t yh = (uint32_t)(y >> 32);
  const int ex = fbias - lz;
  const uint32_t s32 = (uint32_t)sgn & 0x80000000u;
  const uint32_t hb = (((uint32_t)(ex - 1)) << 23) + (yh >> 8);
  const uint32_t nxt = (uint32_t)(y >> 17) & 0x7FFFFFu;
  const uint32_t eb = ((uint32_t)(ex - 23)) << 23;
  auto as_f = [](uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
  };
  auto as_u = [](float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
  };
  const float l = as_f(eb | nxt) - as_f(eb);
  hi = as_f(hb | s32);
  lo = as_f(as_u(l) ^ s32);
}

// One permanent request.  Returns kOk and either fills `hs` (needs_sweep = true)
// or sets `value` directly for the edge cases theboss special-cases.
int plan_permanent(const double* U, int m, const int32_t* S, const int32_t* T, int len, int variant,
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
      bool outs = co < ci;
      st = outs ? fill_sweep(hs, out, in, kGlynn, true, entry_out_in) : fill_sweep(hs, in, out, kGlynn, true, entry_in_out);
      if (st == kErrLimit) {  // try the other orientation
        outs = !outs;
        st = outs ? fill_sweep(hs, out, in, kGlynn, true, entry_out_in) : fill_sweep(hs, in, out, kGlynn, true, entry_in_out);
      }
      if (st) return st;
      hs.digits_are_outputs = outs;
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
  if (in.modes.size() > (size_t)kMaxMinorDigits || out.n > kMaxFactors) {
    set_error("all-minors sweep exceeds 32 distinct input modes or 32 output particles");
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
  // Glynn form: the coefficients of an appended row of variables (every S_i minor_i
  // from one sweep, one single-occupied digit held at r = 0); the kernel
  // accumulates half of each, hence the factor 2.
  auto entry = [&](int i_mode, int j_mode) { return U_at(U, m, j_mode, i_mode); };
  const int st = fill_sweep(hs, in, out, kGlynn, true, entry);
  if (st) return st;
  hs.scale *= 2.0;
  needs_sweep = true;
  return kOk;
}

}  // namespace boss

using namespace boss;

extern "C" {

const char* boss_last_error(void) { return g_last_error.c_str(); }

int boss_abi_version(void) { return BOSS_ABI_VERSION; }

int boss_select_device(int32_t device) {
  std::lock_guard<std::mutex> lk(g_api_mutex);
  if (g_ctx.ready) {
    if (g_ctx.device == device) return kOk;
    set_error("the library's context is already bound to another device");
    return kErrArg;
  }
  cudaError_t e = cudaSetDevice(device);
  return e == cudaSuccess ? kOk : fail_cuda(e, "cudaSetDevice");
}

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
  std::vector<HostSweep> by_nf[kMaxFactors + 1];
  std::vector<int> which[kMaxFactors + 1];
  std::vector<int> small[kSmallPermMax + 1];  // one GPU thread per permanent, no planning
  bool any = false, any_small = false;
  if (variant < BOSS_RYSER || variant > BOSS_CLASSIC) {
    set_error("unknown permanent variant");
    return kErrArg;
  }
  for (int k = 0; k < count; ++k) {
    const int32_t* Sk = input_states + (size_t)k * len;
    const int32_t* Tk = output_states + (size_t)k * len;
    if (len <= m) {  // equal particle counts up to kSmallPermMax: every variant is the permanent
      int ni = 0, no = 0;
      bool ok = true;
      for (int i = 0; i < len; ++i) {
        ok &= (Sk[i] >= 0 && Tk[i] >= 0 && Sk[i] <= 255 && Tk[i] <= 255);
        ni += Sk[i];
        no += Tk[i];
      }
      if (ok && ni == no && ni >= 1 && ni <= kSmallPermMax) {
        small[ni].push_back(k);
        any_small = true;
        continue;
      }
    }
    HostSweep hs;
    bool need = false;
    double2 v = make_double2(0.0, 0.0);
    const int st = plan_permanent(matrix, m, Sk, Tk, len, variant, hs, need, v);
    if (st) return st;
    if (need) {
      which[hs.nf].push_back(k);
      by_nf[hs.nf].push_back(std::move(hs));
      any = true;
    } else {
      results[2 * k] = v.x;
      results[2 * k + 1] = v.y;
    }
  }
  if (!any && !any_small) return kOk;
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  if (any_small && (st = small_perm_batch(cx, matrix, m, len, input_states, output_states, small,
                                          (double2*)results)))
    return st;
  for (int nf = 1; nf <= kMaxFactors; ++nf) {
    if (by_nf[nf].empty()) continue;
    std::vector<double2> out(by_nf[nf].size());
    st = run_sweeps(cx, by_nf[nf], false, 1, out.data());
    if (st) return st;
    for (size_t a = 0; a < out.size(); ++a) {
      results[2 * which[nf][a]] = out[a].x;
      results[2 * which[nf][a] + 1] = out[a].y;
    }
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
  std::vector<HostSweep> by_nf[kMaxFactors + 1];
  std::vector<int> which[kMaxFactors + 1];
  double2* res = (double2*)results;
  bool any = false;
  for (int k = 0; k < count; ++k) {
    HostSweep hs;
    bool need = false;
    const int st = plan_minors(matrix, m, input_states + (size_t)k * len, output_states + (size_t)k * len, len, hs,
                               need, res + (size_t)k * len);
    if (st) return st;
    if (need) {
      which[hs.nf].push_back(k);
      by_nf[hs.nf].push_back(std::move(hs));
      any = true;
    }
  }
  if (!any) return kOk;
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  const int nd_max = kMaxMinorDigits;
  for (int nf = 1; nf <= kMaxFactors; ++nf) {
    if (by_nf[nf].empty()) continue;
    std::vector<double2> out(by_nf[nf].size() * nd_max);
    st = run_sweeps(cx, by_nf[nf], true, nd_max, out.data());
    if (st) return st;
    for (size_t a = 0; a < by_nf[nf].size(); ++a) {
      const HostSweep& hs = by_nf[nf][a];
      double2* row = res + (size_t)which[nf][a] * len;
      for (int d = 0; d < hs.nd; ++d) {  // the sweep gives S_i minor_i
        const double2 v = out[a * nd_max + d];
        row[hs.digit_mode[d]] = make_double2(v.x / hs.mult[d], v.y / hs.mult[d]);
      }
      if (hs.fixed_mode >= 0) row[hs.fixed_mode] = out[a * nd_max + hs.nd];  // the held digit (S_i = 1)
    }
  }
  return kOk;
}

int boss_perm_grad_batch(const double* matrix, int32_t m, const int32_t* input_states,
                         const int32_t* output_states, int32_t len, int32_t count, double* perms, double* grads) {
  if (!matrix || !input_states || !output_states || !perms || !grads || m <= 0 || count < 0 || len <= 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  double2* P2 = (double2*)perms;
  double2* G2 = (double2*)grads;
  std::fill(G2, G2 + (size_t)count * len * len, make_double2(0.0, 0.0));
  std::vector<HostSweep> by_nf[kMaxFactors + 1];
  std::vector<int> which[kMaxFactors + 1];
  bool any = false;
  for (int k = 0; k < count; ++k) {
    HostSweep hs;
    bool need = false;
    double2 v = make_double2(0.0, 0.0);
    const int32_t* S = input_states + (size_t)k * len;
    const int32_t* T = output_states + (size_t)k * len;
    int st = plan_permanent(matrix, m, S, T, len, BOSS_GLYNN, hs, need, v);
    if (st) return st;
    if (!need) {  // no particles: perm = 1, gradient 0
      P2[k] = v;
      continue;
    }
    if (hs.nd + 1 > kMaxDigits) {
      set_error("gradient sweep exceeds the digit limit");
      return kErrLimit;
    }
    which[hs.nf].push_back(k);
    by_nf[hs.nf].push_back(std::move(hs));
    any = true;
  }
  if (!any) return kOk;
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  for (int nf = 1; nf <= kMaxFactors; ++nf) {
    const std::vector<HostSweep>& sw = by_nf[nf];
    const int n = (int)sw.size();
    if (n == 0) continue;
    // at least 32 codes per thread (each thread also writes a (nd+1) x nf slice)
    std::vector<uint64_t> codes(n);
    double total = 0.0;
    for (int p = 0; p < n; ++p) {
      codes[p] = sw[p].total_codes;
      total += (double)codes[p];
    }
    const int64_t resident = sweep_resident_threads(nf, SweepOp::kGrad, cx->sm_count);
    const int64_t want = std::max<int64_t>(n, std::min<int64_t>(resident, (int64_t)(total / 32.0)));
    // whole groups of 32 threads per sweep (the gradient slices interleave by lane),
    // rounded down so the launch stays within one wave of resident threads
    std::vector<int64_t> nthr(n);
    for (int p = 0; p < n; ++p) {
      const int64_t t = (int64_t)std::floor(want * (double)codes[p] / total);
      nthr[p] = std::max<int64_t>(32, t / 32 * 32);
    }
    std::vector<SweepProblem> probs(n);
    int64_t pool_n = 0, threads = 0, gparts = 0;
    int row = 0;
    for (int p = 0; p < n; ++p) row = std::max(row, (sw[p].nd + 1) * nf);
    for (int p = 0; p < n; ++p) {
      const HostSweep& h = sw[p];
      SweepProblem& Pp = probs[p];
      memset(&Pp, 0, sizeof(Pp));
      Pp.nd = h.nd;
      Pp.nb = h.nb;
      Pp.nf = h.nf;
      Pp.kind = h.kind;
      Pp.parity0 = h.parity0;
      Pp.fx = h.fx;
      Pp.has_base = h.has_base;
      Pp.out_idx = p;
      Pp.n_codes = (int64_t)h.total_codes;
      Pp.thread_begin = threads;
      Pp.n_threads = nthr[p];
      Pp.mat_off = pool_n;
      pool_n += (int64_t)h.D.size();
      Pp.base_off = pool_n;
      pool_n += (int64_t)h.base.size();
      Pp.fixed_digit = (h.fixed_mode >= 0) ? 1 : 0;
      Pp.part_off = gparts;
      Pp.scale = h.scale;
      for (int i = 0; i < h.nd; ++i) Pp.mult[i] = h.mult[i];
      threads += nthr[p];
      gparts += nthr[p] * (int64_t)(h.nd + Pp.fixed_digit) * nf;  // nthr is a multiple of 32
    }
    size_t off = 0;
    const size_t o_probs = off; off = align_up(off + sizeof(SweepProblem) * n, 256);
    const size_t o_pool = off; off = align_up(off + sizeof(longlong2) * std::max<int64_t>(pool_n, 1), 256);
    const size_t arena_bytes = off;
    const size_t out_g = (size_t)n * row, out_p = (size_t)n;
    if ((st = ensure(cx->plans, arena_bytes))) return st;
    if ((st = ensure(cx->gpart, sizeof(double2) * std::max<int64_t>(gparts, 1)))) return st;
    if ((st = ensure(cx->pperm, sizeof(double2) * std::max<int64_t>(threads, 1)))) return st;
    if ((st = ensure(cx->out, sizeof(double2) * (out_g + out_p)))) return st;
    if ((st = ensure_pinned(cx, std::max(arena_bytes, sizeof(double2) * (out_g + out_p))))) return st;
    char* h = (char*)cx->pinned;
    memcpy(h + o_probs, probs.data(), sizeof(SweepProblem) * n);
    longlong2* hp = (longlong2*)(h + o_pool);
    for (int p = 0; p < n; ++p) {
      std::copy(sw[p].D.begin(), sw[p].D.end(), hp + probs[p].mat_off);
      std::copy(sw[p].base.begin(), sw[p].base.end(), hp + probs[p].base_off);
    }
    char* d = (char*)cx->plans.ptr;
    cudaError_t e = cudaMemcpyAsync(d, h, arena_bytes, cudaMemcpyHostToDevice, cx->stream);
    if (e != cudaSuccess) return fail_cuda(e, "H2D gradient sweeps");
    SweepLaunch L;
    L.probs = (const SweepProblem*)(d + o_probs);
    L.n_probs = n;
    L.pool = (const longlong2*)(d + o_pool);
    L.total_threads = threads;
    L.partials = (double2*)cx->gpart.ptr;
    L.partials2 = (double2*)cx->pperm.ptr;
    L.grid = (int)((threads + 63) / 64);
    if ((e = launch_sweep(nf, SweepOp::kGrad, L, cx->stream)) != cudaSuccess) return fail_cuda(e, "gradient sweep");
    double2* dout = (double2*)cx->out.ptr;
    if ((e = launch_grad_reduce(L.probs, n, L.partials, L.partials2, dout, dout + out_g, row, cx->stream)) !=
        cudaSuccess)
      return fail_cuda(e, "gradient reduce");
    e = cudaMemcpyAsync(cx->pinned, dout, sizeof(double2) * (out_g + out_p), cudaMemcpyDeviceToHost, cx->stream);
    if (e != cudaSuccess) return fail_cuda(e, "D2H gradients");
    if ((e = cudaStreamSynchronize(cx->stream)) != cudaSuccess) return fail_cuda(e, "gradient sweep");
    const double2* hg = (const double2*)cx->pinned;
    const double2* hpm = hg + out_g;
    for (int p = 0; p < n; ++p) {
      const HostSweep& hs = sw[p];
      const int k = which[nf][p];
      P2[k] = hpm[p];
      double2* gk = G2 + (size_t)k * len * len;
      const int ndt = hs.nd + (hs.fixed_mode >= 0 ? 1 : 0);
      for (int b = 0; b < ndt; ++b) {
        const int bmode = (b < hs.nd) ? hs.digit_mode[b] : hs.fixed_mode;
        for (int f = 0; f < nf; ++f) {
          const int fmode = hs.factor_mode[f];
          const int j = hs.digits_are_outputs ? bmode : fmode;  // output mode
          const int i = hs.digits_are_outputs ? fmode : bmode;  // input mode
          const double2 v = hg[(size_t)p * row + (size_t)b * nf + f];
          gk[(size_t)j * len + i].x += v.x;
          gk[(size_t)j * len + i].y += v.y;
        }
      }
    }
  }
  return kOk;
}

int boss_perm_bench(const double* matrix, int32_t m, const int32_t* input_states, const int32_t* output_states,
                    int32_t len, int32_t count, int32_t variant, int32_t n_warmup, int32_t n_steps,
                    int64_t flush_bytes, double* sweep_ms, double* info, double* results) {
  if (!matrix || !input_states || !output_states || m <= 0 || count <= 0 || n_steps <= 0 || !sweep_ms || !info) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  std::vector<HostSweep> sweeps;
  double flops = 0.0;
  for (int k = 0; k < count; ++k) {
    HostSweep hs;
    bool need = false;
    double2 v;
    const int st = plan_permanent(matrix, m, input_states + (size_t)k * len, output_states + (size_t)k * len, len,
                                  variant, hs, need, v);
    if (st) return st;
    if (!need) {
      set_error("benchmark permanents must need a sweep");
      return kErrArg;
    }
    if (!sweeps.empty() && hs.nf != sweeps[0].nf) {
      set_error("benchmark permanents must share one product size");
      return kErrArg;
    }
    // per code: nf complex adds, nf - 1 complex products, one signed complex add
    flops += (double)hs.total_codes * (8.0 * hs.nf - 4.0);
    sweeps.push_back(std::move(hs));
  }
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  SweepBatch B;
  if ((st = sweeps_prepare(cx, sweeps, false, 1, B))) return st;
  if (flush_bytes > 0 && (st = ensure(cx->misc, (size_t)flush_bytes))) return st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaError_t e = cudaSuccess;
  for (int it = 0; it < n_warmup + n_steps && !st; ++it) {
    if (flush_bytes > 0) e = cudaMemsetAsync(cx->misc.ptr, it & 0xff, (size_t)flush_bytes, cx->stream);
    if (e != cudaSuccess) break;
    cudaEventRecord(e0, cx->stream);
    st = sweeps_launch(cx, B, e1);
    if (st) break;
    e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) break;
    if (it >= n_warmup) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      sweep_ms[it - n_warmup] = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (!st && e != cudaSuccess) st = fail_cuda(e, "perm bench");
  if (st) return st;
  std::vector<double2> out(B.out_elems);
  if ((st = sweeps_collect(cx, B, out.data()))) return st;
  if (results)
    for (int k = 0; k < count; ++k) {
      results[2 * k] = out[k].x;
      results[2 * k + 1] = out[k].y;
    }
  info[0] = B.codes;
  info[1] = flops;
  info[2] = (double)B.L.total_threads;
  info[3] = (double)B.nf;
  // float pairs: nf - 1 renormalised complex products of 38, one complex sum of
  // 16, 15/16 of the codes 16 per factor to move the sums, 1/16 of them 2 per factor
  info[4] = B.ff ? B.codes * (53.125 * B.nf - 22.0) : 0.0;
  return kOk;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free permanents.
//
// Some callers cannot let a library call cudaMalloc: processes that hand all of
// the GPU's memory to their own pool allocator up front and must account for
// every byte, services running under a hard memory cap where a surprise
// allocation can fail or fragment the pool, and latency-sensitive loops that
// avoid cudaMalloc's implicit device synchronisation.  For them
// boss_perm_batch_noalloc runs the same permanent sweep as boss_perm_batch with
// all of its scratch (sweep descriptors, fixed-point rows, per-thread partial
// sums) in one statically sized device array, g_noalloc_scratch below, and
// writes the results into a device buffer the caller owns.
// ---------------------------------------------------------------------------
namespace boss {

constexpr size_t kNoAllocScratchBytes = (size_t)8 << 20;  // 8 MiB, held by every GPU that loads the library
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];
// Host-side copy source, page-locked once (cudaHostRegister: no device memory) so
// that its copies are truly asynchronous; an event recorded after each copy is
// waited on before the array is refilled.
alignas(4096) static unsigned char g_noalloc_staging[kNoAllocScratchBytes];
static bool g_noalloc_staging_pinned = false;
static cudaEvent_t g_noalloc_staging_free = nullptr;  // recorded after the last copy out of the staging array

struct NoAllocDevice {
  bool ready = false;
  int sm_count = 0;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch on this device
  cudaEvent_t copied = nullptr;      // this device's staging-copy event
};
constexpr int kNoAllocMaxDevices = 64;
static NoAllocDevice g_noalloc_dev[kNoAllocMaxDevices];

// Once per device, with that device current: the device address of the scratch
// array (its host-side name is only a stand-in), the kernel attributes and the
// staging-copy event; once per process, the staging array is page-locked.
static int noalloc_setup(int device, NoAllocDevice*& out) {
  if (device < 0 || device >= kNoAllocMaxDevices) {
    set_error("device index out of range");
    return kErrArg;
  }
  NoAllocDevice& d = g_noalloc_dev[device];
  if (!d.ready) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return fail_cuda(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    if ((e = cudaDeviceGetAttribute(&d.sm_count, cudaDevAttrMultiProcessorCount, device)) != cudaSuccess)
      return fail_cuda(e, "cudaDeviceGetAttribute");
    if ((e = prepare_sweep_kernels()) != cudaSuccess) return fail_cuda(e, "kernel attributes");
    if ((e = cudaEventCreateWithFlags(&d.copied, cudaEventDisableTiming)) != cudaSuccess)
      return fail_cuda(e, "cudaEventCreate");
    if (!g_noalloc_staging_pinned) {
      e = cudaHostRegister(g_noalloc_staging, sizeof(g_noalloc_staging), cudaHostRegisterPortable);
      if (e != cudaSuccess) return fail_cuda(e, "cudaHostRegister(staging)");
      g_noalloc_staging_pinned = true;
    }
    d.scratch = (unsigned char*)p;
    d.ready = true;
  }
  out = &d;
  return kOk;
}

// Waits until the staging array's last copy has left it (from any device).
static int noalloc_staging_wait() {
  if (!g_noalloc_staging_free) return kOk;
  cudaError_t e = cudaEventSynchronize(g_noalloc_staging_free);
  return e == cudaSuccess ? kOk : fail_cuda(e, "staging copy");
}

// Queues the copy of the first `bytes` of the staging array into the device's
// scratch and marks the staging array busy until it has left.
static int noalloc_stage(NoAllocDevice* dev, size_t bytes, cudaStream_t s) {
  cudaError_t e = cudaMemcpyAsync(dev->scratch, g_noalloc_staging, bytes, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail_cuda(e, "H2D staging");
  if ((e = cudaEventRecord(dev->copied, s)) != cudaSuccess) return fail_cuda(e, "event record");
  g_noalloc_staging_free = dev->copied;
  return kOk;
}

// Results that need no sweep (theboss's empty-state rules): out[idx[i]] = val[i].
__global__ void noalloc_scatter_kernel(const int32_t* __restrict__ idx, const double2* __restrict__ val, int n,
                                       double2* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[idx[i]] = val[i];
}

// One product-size group of a request: its sweeps' layout in the scratch.
struct NoAllocGroup {
  int nf = 0;
  std::vector<int64_t> nthr;
  int64_t threads = 0;
  size_t o_pool = 0, o_part = 0, bytes = 0;
};

}  // namespace boss

extern "C" int boss_perm_batch_noalloc(const double* matrix, int32_t m, const int32_t* input_states,
                                       const int32_t* output_states, int32_t len, int32_t count, int32_t variant,
                                       double* results_device, void* stream) {
  if (!matrix || !input_states || !output_states || !results_device || m <= 0 || count < 0) {
    set_error("null pointer or bad size");
    return kErrArg;
  }
  std::lock_guard<std::mutex> lk(g_api_mutex);
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return fail_cuda(e, "cudaGetDevice");
  NoAllocDevice* dev = nullptr;
  int st = noalloc_setup(device, dev);
  if (st) return st;
  cudaStream_t s = (cudaStream_t)stream;
  double2* out = (double2*)results_device;
  // (1) Plan every permanent and lay out every scratch image; reject the request
  // before anything is queued if one image exceeds the scratch.
  std::vector<HostSweep> by_nf[kMaxFactors + 1];
  std::vector<int> which[kMaxFactors + 1];
  std::vector<int32_t> direct_idx;
  std::vector<double2> direct_val;
  for (int k = 0; k < count; ++k) {
    HostSweep hs;
    bool need = false;
    double2 v = make_double2(0.0, 0.0);
    st = plan_permanent(matrix, m, input_states + (size_t)k * len, output_states + (size_t)k * len, len, variant, hs,
                        need, v);
    if (st) return st;
    if (need) {
      which[hs.nf].push_back(k);
      by_nf[hs.nf].push_back(std::move(hs));
    } else {  // a permanent theboss defines without a sweep (empty states)
      direct_idx.push_back(k);
      direct_val.push_back(v);
    }
  }
  const size_t o_dval = align_up(sizeof(int32_t) * direct_idx.size(), 256);
  const size_t direct_bytes = o_dval + sizeof(double2) * direct_val.size();
  std::vector<NoAllocGroup> groups;
  for (int nf = 1; nf <= kMaxFactors; ++nf) {
    const std::vector<HostSweep>& sw = by_nf[nf];
    const int n = (int)sw.size();
    if (n == 0) continue;
    NoAllocGroup G;
    G.nf = nf;
    std::vector<uint64_t> codes(n);
    for (int p = 0; p < n; ++p) codes[p] = sw[p].total_codes;
    partition_threads(codes, sweep_resident_threads(nf, SweepOp::kPerm, dev->sm_count), G.nthr);
    int64_t pool_n = 0;
    for (int p = 0; p < n; ++p) {
      pool_n += (int64_t)(sw[p].D.size() + sw[p].base.size());
      G.threads += G.nthr[p];
    }
    G.o_pool = align_up(sizeof(SweepProblem) * n, 256);
    G.o_part = align_up(G.o_pool + sizeof(longlong2) * (size_t)std::max<int64_t>(pool_n, 1), 256);
    G.bytes = G.o_part + sizeof(double2) * (size_t)G.threads;
    groups.push_back(std::move(G));
  }
  size_t need_bytes = direct_bytes;
  for (const NoAllocGroup& G : groups) need_bytes = std::max(need_bytes, G.bytes);
  if (need_bytes > kNoAllocScratchBytes) {
    set_error("request needs " + std::to_string(need_bytes) + " bytes of scratch; the allocation-free entry "
              "point has " + std::to_string(kNoAllocScratchBytes) + " (split the batch)");
    return kErrLimit;
  }
  // (2) The direct results, through the staging array and a scatter kernel.
  if (!direct_idx.empty()) {
    if ((st = noalloc_staging_wait())) return st;
    memcpy(g_noalloc_staging, direct_idx.data(), sizeof(int32_t) * direct_idx.size());
    memcpy(g_noalloc_staging + o_dval, direct_val.data(), sizeof(double2) * direct_val.size());
    if ((st = noalloc_stage(dev, direct_bytes, s))) return st;
    const int nd = (int)direct_idx.size();
    noalloc_scatter_kernel<<<(nd + 127) / 128, 128, 0, s>>>((const int32_t*)dev->scratch,
                                                            (const double2*)(dev->scratch + o_dval), nd, out);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail_cuda(e, "scatter launch");
  }
  // (3) One sweep launch per product size; each image reuses the scratch from its
  // start (stream order keeps it behind the previous image's kernels).
  for (const NoAllocGroup& G : groups) {
    const int nf = G.nf;
    const std::vector<HostSweep>& sw = by_nf[nf];
    const int n = (int)sw.size();
    if ((st = noalloc_staging_wait())) return st;
    SweepProblem* hp = (SweepProblem*)g_noalloc_staging;
    longlong2* hpool = (longlong2*)(g_noalloc_staging + G.o_pool);
    int64_t pool_at = 0, thread_at = 0;
    for (int p = 0; p < n; ++p) {
      const HostSweep& h = sw[p];
      SweepProblem& P = hp[p];
      memset(&P, 0, sizeof(P));
      P.nd = h.nd;
      P.nb = h.nb;
      P.nf = h.nf;
      P.kind = h.kind;
      P.parity0 = h.parity0;
      P.fx = h.fx;
      P.has_base = h.has_base;
      P.out_idx = which[nf][p];  // the reduction writes straight into the caller's buffer
      P.n_codes = (int64_t)h.total_codes;
      P.thread_begin = thread_at;
      P.n_threads = G.nthr[p];
      P.mat_off = pool_at;
      std::copy(h.D.begin(), h.D.end(), hpool + pool_at);
      pool_at += (int64_t)h.D.size();
      P.base_off = pool_at;
      std::copy(h.base.begin(), h.base.end(), hpool + pool_at);
      pool_at += (int64_t)h.base.size();
      P.part_off = thread_at;
      P.scale = h.scale;
      for (int i = 0; i < h.nd; ++i) P.mult[i] = h.mult[i];
      thread_at += G.nthr[p];
    }
    if ((st = noalloc_stage(dev, G.o_part, s))) return st;
    SweepLaunch L;
    L.probs = (const SweepProblem*)dev->scratch;
    L.n_probs = n;
    L.pool = (const longlong2*)(dev->scratch + G.o_pool);
    L.total_threads = G.threads;
    L.partials = (double2*)(dev->scratch + G.o_part);
    L.grid = (int)((G.threads + 127) / 128);
    if ((e = launch_sweep(nf, SweepOp::kPerm, L, s)) != cudaSuccess) return fail_cuda(e, "sweep launch");
    if ((e = launch_perm_reduce(L.probs, n, L.partials, out, s)) != cudaSuccess) return fail_cuda(e, "reduce launch");
  }
  return kOk;
}
