// boss_internal.h -- declarations shared by the CUDA translation units of
// libboss_gb300.so.  Not part of the public C ABI (that is include/boss.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "boss_sweep.cuh"

namespace boss {

// Everything one sweep launch needs (device pointers).
struct SweepLaunch {
  const SweepPlan* plans = nullptr;
  int n_plans = 0;
  const double2* pool = nullptr;
  int64_t total_items = 0;
  unsigned long long* counter = nullptr;  // zeroed before the launch
  double2* partials = nullptr;
  int max_nc = 1;
  int grid = 1;
};

cudaError_t prepare_sweep_kernels();
cudaError_t launch_perm_sweep(const SweepLaunch& L, cudaStream_t st);
cudaError_t launch_minors_sweep(const SweepLaunch& L, cudaStream_t st);
cudaError_t launch_perm_reduce(const SweepPlan* plans, const int32_t* out_plans, const int32_t* out_begin, int n_out,
                               const double2* partials, double2* out, cudaStream_t st);
cudaError_t launch_minors_reduce(const SweepPlan* plans, const int32_t* out_plans, const int32_t* out_begin,
                                 int n_out, const double2* partials, double2* out, int nd_max, cudaStream_t st);

// ---------------------------------------------------------------------------
// Host-side sweep description before it is cut into segments.
// ---------------------------------------------------------------------------
struct HostSweep {
  int kind = kRyser;
  int parity0 = 0;
  int nd = 0, nb = 0, nc = 0;
  int has_base = 0;
  uint8_t mult[kMaxDigits] = {};
  uint8_t pw[kMaxCols] = {};
  std::vector<double2> D;     // nd x nc
  std::vector<double2> base;  // nc (has_base)
  double scale = 1.0;
  uint64_t total_codes = 1;
  int digit_mode[kMaxDigits] = {};  // digit -> mode (all-minors results)
};

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

// Per-process device context: one non-blocking stream, SM count, grow-only buffers.
struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
};
struct Context {
  bool ready = false;
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  DeviceBuffer plans, pool, partials, out, counter, index, misc;
  DeviceBuffer gccb[16];
  void* pinned = nullptr;
  size_t pinned_bytes = 0;
};
Context* context(int* status);
int ensure(DeviceBuffer& b, size_t bytes);
int ensure_pinned(Context* cx, size_t bytes);

// Builds the segments of a list of sweeps into device plan arrays and launches
// sweep + reduction.  results: n_out complex (perms) or n_out x nd_max (minors).
int run_sweeps(Context* cx, const std::vector<HostSweep>& sweeps, bool minors, int nd_max, double2* results_host);

}  // namespace boss
