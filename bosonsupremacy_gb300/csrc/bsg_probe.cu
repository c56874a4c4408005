// Measurement helper: FMA throughput of the CUDA cores (FP64 or FP32).
// Eight independent register chains per thread keep the pipe busy; the
// result is stored only if it is NaN so the loop cannot be removed.
#include "bsg_internal.h"

namespace bsg {

template <class T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T seed, int iters, T* sink) {
  T a0 = seed + T(threadIdx.x) * T(1e-7), a1 = a0 + T(1e-3), a2 = a0 + T(2e-3), a3 = a0 + T(3e-3);
  T a4 = a0 + T(4e-3), a5 = a0 + T(5e-3), a6 = a0 + T(6e-3), a7 = a0 + T(7e-3);
  const T b = T(0.999999), c = T(1e-6);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = a0 * b + c;
      a1 = a1 * b + c;
      a2 = a2 * b + c;
      a3 = a3 * b + c;
      a4 = a4 * b + c;
      a5 = a5 * b + c;
      a6 = a6 * b + c;
      a7 = a7 * b + c;
    }
  }
  T s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s != s) sink[blockIdx.x] = s;
}

}  // namespace bsg

using namespace bsg;

extern "C" int bsg_fma_peak(bsg_handle_t h, int precision, double* flops_per_s, bsg_stream_t stream) {
  BSG_CHECK_ARG(h && flops_per_s, "bsg_fma_peak: null pointer");
  BSG_CHECK_ARG(precision == BSG_PREC_FP64 || precision == BSG_PREC_FP32, "bsg_fma_peak: FP64 or FP32 only");
  BSG_CUDA(cudaSetDevice(h->device));
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  BSG_TRY(h->misc.ensure(4096 * 8));
  const int blocks = h->num_sms * 8, threads = 256;
  const int iters = precision == BSG_PREC_FP64 ? 256 : 8192;
  cudaEvent_t e0, e1;
  BSG_CUDA(cudaEventCreate(&e0));
  BSG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  for (int rep = 0; rep < 4; ++rep) {
    BSG_CUDA(cudaEventRecord(e0, st));
    if (precision == BSG_PREC_FP64)
      fma_probe_kernel<double><<<blocks, threads, 0, st>>>(1.0, iters, reinterpret_cast<double*>(h->misc.ptr));
    else
      fma_probe_kernel<float><<<blocks, threads, 0, st>>>(1.0f, iters, reinterpret_cast<float*>(h->misc.ptr));
    BSG_CUDA(cudaGetLastError());
    BSG_CUDA(cudaEventRecord(e1, st));
    BSG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    BSG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && ms < best) best = ms;  // first launch is warm-up
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  const double fmas = (double)blocks * threads * iters * 16.0 * 8.0;
  *flops_per_s = 2.0 * fmas / (best * 1e-3);
  return BSG_OK;
}
