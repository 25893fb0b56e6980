// Peak rates of the FP64 units of the current device: fused multiply-adds
// and IEEE double divisions, each as many independent chains per thread as
// keep the pipe full, over a grid of 16 blocks per SM. These are the
// denominators of the FP64 form's bound: its kernels keep the FP64 pipe
// 84-87 % busy (ncu sm__pipe_fp64_cycles_active) while DRAM runs far below
// its bandwidth.
#include <cuda_runtime.h>

#include <string>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"

namespace {

constexpr int kChainsFma = 8, kChainsDiv = 4, kThreads = 256, kBlocksPerSM = 16;

__global__ void __launch_bounds__(kThreads) k_probe_fma64(double* sink, int iters, double a, double b) {
  double x[kChainsFma];
#pragma unroll
  for (int c = 0; c < kChainsFma; ++c) x[c] = 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChainsFma; ++c) x[c] = fma(x[c], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChainsFma; ++c) s += x[c];
  if (s == -1.0) sink[0] = s;  // never true (every chain stays near 1): keeps the chains live
}

__global__ void __launch_bounds__(kThreads) k_probe_div64(double* sink, int iters, double a) {
  double x[kChainsDiv];
#pragma unroll
  for (int c = 0; c < kChainsDiv; ++c) x[c] = 1.25 + 1e-3 * (threadIdx.x + c);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < kChainsDiv; ++c) x[c] = a / x[c];  // alternates between x0 and a / x0
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < kChainsDiv; ++c) s += x[c];
  if (s == -1.0) sink[0] = s;
}

}  // namespace

extern "C" int fgb_probe_fp64(double* out3, void* stream) {
  if (!out3) {
    fgb::set_error("fgb_probe_fp64: null argument");
    return -1;
  }
  auto fail = [](const char* what, cudaError_t e) {
    fgb::set_error(std::string("fgb_probe_fp64: ") + what + ": " + cudaGetErrorString(e));
    return -1;
  };
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return fail("device query", e);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* sink = nullptr;
  cudaEvent_t ev[4] = {};
  if ((e = cudaMallocAsync(reinterpret_cast<void**>(&sink), sizeof(double), s)) != cudaSuccess)
    return fail("cudaMallocAsync", e);
  for (auto& x : ev)
    if (e == cudaSuccess) e = cudaEventCreate(&x);
  const int blocks = sms * kBlocksPerSM, it_fma = 4096, it_div = 512;
  if (e == cudaSuccess) {
    // warm-up launches (clocks, module load), then the timed ones
    k_probe_fma64<<<blocks, kThreads, 0, s>>>(sink, 64, 0.9999999, 1e-7);
    k_probe_div64<<<blocks, kThreads, 0, s>>>(sink, 16, 1.7);
    cudaEventRecord(ev[0], s);
    k_probe_fma64<<<blocks, kThreads, 0, s>>>(sink, it_fma, 0.9999999, 1e-7);
    cudaEventRecord(ev[1], s);
    cudaEventRecord(ev[2], s);
    k_probe_div64<<<blocks, kThreads, 0, s>>>(sink, it_div, 1.7);
    cudaEventRecord(ev[3], s);
    e = cudaEventSynchronize(ev[3]);
  }
  float ms_fma = 0.f, ms_div = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms_fma, ev[0], ev[1]);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms_div, ev[2], ev[3]);
  for (auto& x : ev)
    if (x) cudaEventDestroy(x);
  cudaError_t ef = cudaFreeAsync(sink, s);
  if (e == cudaSuccess) e = ef;
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail("probe launch", e);
  const double threads = double(blocks) * kThreads;
  out3[0] = threads * it_fma * kChainsFma * 2.0 / (ms_fma * 1e-3) / 1e12;  // TFLOP/s (an FMA is 2 flops)
  out3[1] = threads * it_div * kChainsDiv / (ms_div * 1e-3) / 1e9;        // G divisions/s
  out3[2] = double(ms_fma) + double(ms_div);
  return 0;
}
