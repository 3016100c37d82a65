// gbh_probe.cu -- probes of the hardware the fused kernels rely on.
//
// gb_probe_fp64_peak: FP64 FMA throughput, the denominator of the FP64-pipe
// roofline reported next to the fused kernels (the chip's measured DFMA rate,
// not a datasheet figure).  Eight independent FMA chains per thread, all
// operands in registers, enough blocks to fill every SM several times.
//
// gb_probe_rcp_sqrt: the Newton-Raphson reciprocal and square root of
// gbh_device.cuh next to CUDA's correctly rounded 1.0/x and sqrt(x) on the same
// inputs, so that their error bound can be checked directly.
#include <cuda_runtime.h>

#include "gbh_device.cuh"
#include "gbhypar.h"

extern "C" void gbh_set_error(const char* fmt, ...);

namespace gbh {
__global__ void dfma_probe_kernel(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1.0, x2 = x0 + 2.0, x3 = x0 + 3.0;
  double x4 = x0 + 4.0, x5 = x0 + 5.0, x6 = x0 + 6.0, x7 = x0 + 7.0;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

__global__ void rcp_sqrt_probe_kernel(const double* __restrict__ x, double* __restrict__ rcp_nr,
                                      double* __restrict__ rcp_ieee, double* __restrict__ sqrt_nr,
                                      double* __restrict__ sqrt_ieee, double* __restrict__ rsqrt_nr,
                                      long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const double v = x[i];
    rcp_nr[i] = nr_rcp(v);
    rcp_ieee[i] = __drcp_rn(v);
    sqrt_nr[i] = nr_sqrt(v);
    sqrt_ieee[i] = __dsqrt_rn(v);
    if (rsqrt_nr) rsqrt_nr[i] = nr_rsqrt(v);
  }
}
}  // namespace gbh

extern "C" int gb_probe_rcp_sqrt(const double* x, double* rcp_nr, double* rcp_ieee, double* sqrt_nr,
                                 double* sqrt_ieee, double* rsqrt_nr, long long n) {
  if (n < 0 || (n > 0 && (!x || !rcp_nr || !rcp_ieee || !sqrt_nr || !sqrt_ieee))) {
    gbh_set_error("gb_probe_rcp_sqrt: null array or negative length");
    return GB_ERR_ARG;
  }
  if (n == 0) return GB_OK;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  long long want = (n + 255) / 256;
  int blocks = (int)(want < (long long)sms * 16 ? want : (long long)sms * 16);
  gbh::rcp_sqrt_probe_kernel<<<blocks, 256>>>(x, rcp_nr, rcp_ieee, sqrt_nr, sqrt_ieee, rsqrt_nr, n);
  cudaError_t e = cudaDeviceSynchronize();
  if (e != cudaSuccess) { gbh_set_error("gb_probe_rcp_sqrt: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
  return GB_OK;
}

extern "C" int gb_probe_fp64_peak(double* tflops) {
  if (!tflops) { gbh_set_error("gb_probe_fp64_peak: null argument"); return GB_ERR_ARG; }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) { gbh_set_error("cudaMalloc failed"); return GB_ERR_CUDA; }
  const int threads = 256, iters = 2048;
  const int blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  gbh::dfma_probe_kernel<<<blocks, threads>>>(out, 64, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  gbh::dfma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (e != cudaSuccess || ms <= 0.f) { gbh_set_error("probe failed: %s", cudaGetErrorString(e)); return GB_ERR_CUDA; }
  double flops = 2.0 * 8.0 * 16.0 * (double)iters * threads * (double)blocks;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return GB_OK;
}
