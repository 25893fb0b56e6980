// Device-side check of a step's inputs: every value of the arrays a step
// reads is finite. One grid-stride reduction per array sets a bit of a
// status word (no assert, no trap: a non-finite value is a result, not a
// fault). The reference has no such check; its arithmetic carries NaN and
// Inf through the step.
#include <cuda_runtime.h>

#include <string>

#include "fesom_tracer_gb300.h"
#include "fgb_internal.hpp"

namespace {

constexpr int kCheckThreads = 256;

template <typename R>
__global__ void __launch_bounds__(kCheckThreads) k_nonfinite(const R* __restrict__ p, long long n, unsigned bit,
                                                              unsigned* flags) {
  bool bad = false;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    bad |= !isfinite(p[i]);
  if (__syncthreads_or(bad) && threadIdx.x == 0) atomicOr(flags, bit);
}

template <typename R>
void check(const void* p, long long n, unsigned bit, unsigned* flags, int blocks, cudaStream_t s) {
  if (!p || n <= 0) return;
  const long long need = (n + kCheckThreads - 1) / kCheckThreads;
  const int grid = (int)(need < blocks ? need : blocks);
  k_nonfinite<R><<<grid, kCheckThreads, 0, s>>>(static_cast<const R*>(p), n, bit, flags);
}

template <typename R>
void check_all(const fgb::DMesh& m, const fgb_step_desc& d, unsigned* flags, int blocks, cudaStream_t s) {
  const int V = (d.precision == FGB_FP32 && d.tracer_vec > 1) ? d.tracer_vec : 1;
  const int G = d.ntracers / V;
  const long long per = (long long)m.N * m.LZ * V;
  const R* T = static_cast<const R*>(d.T);
  for (int g = 0; g < G; ++g) check<R>(T + g * d.strideT, per, FGB_CHECK_T, flags, blocks, s);
  if (d.TA && d.TA != d.T) {
    const R* TA = static_cast<const R*>(d.TA);
    for (int g = 0; g < G; ++g) check<R>(TA + g * d.strideTA, per, FGB_CHECK_TA, flags, blocks, s);
  }
  if (d.precision == FGB_FP32 && d.Tlo) {
    const R* Tlo = static_cast<const R*>(d.Tlo);
    for (int g = 0; g < G; ++g) check<R>(Tlo + g * d.strideT, per, FGB_CHECK_TLO, flags, blocks, s);
  }
  check<R>(d.vel, (long long)m.M * m.LZ * 2, FGB_CHECK_VEL, flags, blocks, s);
  check<R>(d.w, (long long)m.N * m.LW, FGB_CHECK_W, flags, blocks, s);
  if (d.we && d.we != d.w) check<R>(d.we, (long long)m.N * m.LW, FGB_CHECK_WE, flags, blocks, s);
  if (d.wi) check<R>(d.wi, (long long)m.N * m.LW, FGB_CHECK_WI, flags, blocks, s);
}

}  // namespace

extern "C" int fgb_check_inputs(const fgb_mesh* m, const fgb_step_desc* d, void* stream, int* flags_out) {
  if (!m || !d || !flags_out || !d->T || !d->vel || !d->w || d->ntracers < 1) {
    fgb::set_error("fgb_check_inputs: null or empty argument");
    return -1;
  }
  const int V = (d->precision == FGB_FP32 && d->tracer_vec > 1) ? d->tracer_vec : 1;
  if (d->ntracers % V) {
    fgb::set_error("fgb_check_inputs: tracer_vec does not divide ntracers");
    return -1;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int dev = 0, sms = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  unsigned* flags = nullptr;
  if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&flags), sizeof(unsigned), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, sizeof(unsigned), s);
  unsigned host = 0;
  if (e == cudaSuccess) {
    const int blocks = 8 * (sms > 0 ? sms : 1);
    if (d->precision == FGB_FP32) check_all<float>(m->d, *d, flags, blocks, s);
    else check_all<double>(m->d, *d, flags, blocks, s);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(&host, flags, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
  }
  if (flags) {
    cudaError_t ef = cudaFreeAsync(flags, s);
    if (e == cudaSuccess) e = ef;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    fgb::set_error(std::string("fgb_check_inputs: ") + cudaGetErrorString(e));
    return -1;
  }
  *flags_out = (int)host;
  return 0;
}
