// boss_internal.h -- declarations shared by the CUDA translation units of
// libboss_gb300.so.  Not part of the public C ABI (that is include/boss.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "boss_sweep.cuh"

namespace boss {

enum class SweepOp { kPerm = 0, kMinors = 1, kGrad = 2, kMinorsFF = 3, kPermFF = 4 };  // FF: float pairs

// Everything one sweep launch needs (device pointers).
struct SweepLaunch {
  const SweepProblem* probs = nullptr;
  int n_probs = 0;
  const longlong2* pool = nullptr;
  int64_t total_threads = 0;
  double2* partials = nullptr;
  double2* partials2 = nullptr;  // gradients: per-warp permanent partials
  int grid = 1;
  int rows = 32;  // all-minors: shared-memory rows of minors per thread (nd + held digit, at most 32)
  int64_t uniform_threads = 0;  // all-minors: > 0 when every sweep has this many threads and sweep p
                                // starts at thread p * uniform_threads (no search for the sweep)
};

// Sets kernel attributes and records occupancy (once per process, outside any capture).
cudaError_t prepare_sweep_kernels();
// Resident threads of one full wave of the sweep kernel for `nf` factors.
int64_t sweep_resident_threads(int nf, SweepOp op, int sm_count);
// Resident threads of the all-minors kernel (FP64, or the float-pair one) with
// `rows` rows of minors per thread.
int64_t sweep_resident_minors(int nf, int rows, int sm_count, bool ff = false);
// Whether the float-pair all-minors / single-permanent kernel exists for nf factors.
bool minors_ff_available(int nf);
bool perm_ff_available(int nf);
cudaError_t launch_sweep(int nf, SweepOp op, const SweepLaunch& L, cudaStream_t st);
cudaError_t launch_perm_reduce(const SweepProblem* probs, int n_probs, const double2* partials, double2* out,
                               cudaStream_t st, bool ff = false);
cudaError_t launch_grad_reduce(const SweepProblem* probs, int n_probs, const double2* gpart, const double2* ppart,
                               double2* grad_out, double2* perm_out, int row_stride, cudaStream_t st);
cudaError_t launch_minors_reduce(const SweepProblem* probs, int n_probs, const double2* partials, double2* out,
                                 int nd_max, cudaStream_t st, bool ff = false);

// Splits `n_codes` codes over at most `resident` threads, proportionally, at
// least one thread per sweep and at least kMinCodesPerThread codes per thread.
constexpr int64_t kMinCodesPerThread = 8;
void partition_threads(const std::vector<uint64_t>& n_codes, int64_t resident, std::vector<int64_t>& n_threads);

// ---------------------------------------------------------------------------
// Host-side sweep description.
// ---------------------------------------------------------------------------
struct HostSweep {
  int kind = kRyser;
  int parity0 = 0;
  int nd = 0, nb = 0, nf = 0;
  int has_base = 0;
  int fx = 56;
  uint8_t mult[kMaxDigits] = {};
  std::vector<longlong2> D;     // nd x nf
  std::vector<longlong2> base;  // nf (has_base)
  double scale = 1.0;
  uint64_t total_codes = 1;
  int digit_mode[kMaxDigits] = {};  // digit -> mode (all-minors results)
  int factor_mode[kMaxFactors] = {};  // factor -> mode (gradients)
  int fixed_mode = -1;                // mode of the digit held at r = 0 (Glynn halving), or -1
  bool digits_are_outputs = false;    // orientation of the sweep
  // Float-pair all-minors: factor f's bound 2^p <= max(sum mult |Re|, sum mult |Im|) < 2^(p+1)
  // over every digit (held one included), in fixed-point units; fx_to_ff takes 189 - p.
  std::vector<int> fbias;
  int ff_exp = 0;  // sum_f (p_f + 1) - nf * fx: the float-pair products' scale
};

// Arithmetic of the all-minors sweeps (boss_minors_arithmetic): 0 float pairs
// where the kernel exists for the factor count, 1 FP64.
extern int g_minors_arith;
// Arithmetic of the single-permanent sweeps (boss_perm_arithmetic), same codes.
extern int g_perm_arith;
// x * 2^(fbias - 190) as a float pair, the host twin of fx_to_ff (same bits).
void host_fx_to_ff(long long x, int fbias, float& hi, float& lo);

// Status codes of the C ABI (include/boss.h repeats them).
enum Status : int {
  kOk = 0,
  kErrSize = 1,     // size mismatch: theboss raises AttributeError
  kErrLimit = 2,    // beyond this library's limits
  kErrCuda = 3,     // CUDA runtime error
  kErrArg = 4,      // invalid argument
  kErrPmf = 5,      // a pmf could not be normalised (theboss: ValueError in numpy.random.choice)
  kErrNoDevice = 6  // no CUDA device
};

void set_error(const std::string& msg);
int fail_cuda(cudaError_t e, const char* where);

// Per-process device context: non-blocking streams, SM count, grow-only buffers.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};
struct Context {
  bool ready = false;
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t sampler_streams[3] = {nullptr, nullptr, nullptr};  // the sampler's pipelined slots 1..3 (boss_gccb.cu)
  DeviceBuffer plans, pool, partials, out, counter, index, misc, gpart, pperm;
  DeviceBuffer gccb[32];  // the sampler's slots, 8 each
  DeviceBuffer dist[4];
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
};
Context* context(int* status);
int ensure(DeviceBuffer& b, size_t bytes);
int ensure_pinned(Context* cx, size_t bytes);

// Uploads a list of sweeps (all with the same factor count), launches the sweep
// and the reduction, copies the results back.  results: one complex per sweep
// (perms) or nd_max complex per sweep (all-minors).
int run_sweeps(Context* cx, const std::vector<HostSweep>& sweeps, bool minors, int nd_max, double2* results_host);

// Permanents of at most kSmallPermMax particles, one GPU thread each (Glynn's
// formula in registers, no sweep planning): by_l[l] lists the requests k with
// l = sum(S_k) = sum(T_k) particles; S, T are the callers' occupation rows.
constexpr int kSmallPermMax = 10;
int small_perm_batch(Context* cx, const double* matrix, int m, int len, const int32_t* S, const int32_t* T,
                     const std::vector<int>* by_l, double2* results);

// One permanent request (theboss's variant semantics).  Returns kOk and either
// fills `hs` (needs_sweep = true) or sets `value` for the edge cases theboss
// special-cases.
int plan_permanent(const double* U, int m, const int32_t* S, const int32_t* T, int len, int variant, HostSweep& hs,
                   bool& needs_sweep, double2& value);

}  // namespace boss
