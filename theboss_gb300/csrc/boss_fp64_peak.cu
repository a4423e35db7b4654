// boss_fp64_peak.cu -- FP64 and FP32 FMA throughput of the current GPU (the
// denominators of the FP64 roofline and of the float-pair kernels' FP32 roofline).
// Every thread runs 8 independent FMA chains so neither latency nor occupancy
// limits the pipe; the chains' results are stored so the compiler keeps the work.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/boss.h"
#include "boss_internal.h"

namespace boss {

extern std::mutex g_api_mutex;

static __global__ void __launch_bounds__(256) fp64_fma_stream(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = 1e-3 * threadIdx.x + j;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fma(x[j], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

static __global__ void __launch_bounds__(256) fp32_fma_stream(float* out, int iters, float a, float b) {
  float x[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) x[j] = 1e-3f * threadIdx.x + j;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = fmaf(x[j], a, b);
  }
  float s = 0.0f;
#pragma unroll
  for (int j = 0; j < 8; ++j) s += x[j];
  out[(size_t)blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace boss

using namespace boss;

extern "C" int boss_fp32_peak(double* tinst, double* milliseconds) {
  std::lock_guard<std::mutex> lk(g_api_mutex);
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  const int blocks = cx->sm_count * 8, threads = 256, iters = 16384;
  if ((st = ensure(cx->misc, sizeof(float) * blocks * threads))) return st;
  float* out = (float*)cx->misc.ptr;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp32_fma_stream<<<blocks, threads, 0, cx->stream>>>(out, 256, 1.0000001f, 1e-9f);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, cx->stream);
    fp32_fma_stream<<<blocks, threads, 0, cx->stream>>>(out, iters, 1.0000001f, 1e-9f);
    cudaEventRecord(e1, cx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail_cuda(e, "fp32 peak");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double inst = 8.0 * (double)iters * blocks * threads;  // FP32 FMA instructions (per lane)
  *tinst = inst / (best * 1e-3) / 1e12;
  *milliseconds = best;
  return BOSS_OK;
}

extern "C" int boss_fp64_peak(double* tflops, double* milliseconds) {
  std::lock_guard<std::mutex> lk(g_api_mutex);
  int st;
  Context* cx = context(&st);
  if (!cx) return st;
  const int blocks = cx->sm_count * 8, threads = 256, iters = 4096;
  if ((st = ensure(cx->misc, sizeof(double) * blocks * threads))) return st;
  double* out = (double*)cx->misc.ptr;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fp64_fma_stream<<<blocks, threads, 0, cx->stream>>>(out, 64, 1.0000001, 1e-9);  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, cx->stream);
    fp64_fma_stream<<<blocks, threads, 0, cx->stream>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1, cx->stream);
    cudaError_t e = cudaEventSynchronize(e1);
    if (e != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return fail_cuda(e, "fp64 peak");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = ms < best ? ms : best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *tflops = flops / (best * 1e-3) / 1e12;
  *milliseconds = best;
  return BOSS_OK;
}
