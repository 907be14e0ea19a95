// fp64_peak.cu -- measures the FP64 FMA throughput of the device, the
// denominator of the roofline of the FP64-bound Newton kernel.
//
// Each thread runs 8 independent DFMA chains; the grid fills every SM with
// 32 warps.  The result is reported in TFLOP/s with one FMA = 2 flops.
#include <cuda_runtime.h>

#include <cstdint>

namespace {
__global__ void __launch_bounds__(1024) dfma_chains(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      x0 = fma(x0, a, b);
      x1 = fma(x1, a, b);
      x2 = fma(x2, a, b);
      x3 = fma(x3, a, b);
      x4 = fma(x4, a, b);
      x5 = fma(x5, a, b);
      x6 = fma(x6, a, b);
      x7 = fma(x7, a, b);
    }
  }
  const double s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == 1.2345) out[blockIdx.x] = s;  // keeps the chains alive
}
}  // namespace

extern "C" int pfchem_probe_fp64_peak(int device, int iters, double *tflops, double *ms_out) {
  if (cudaSetDevice(device) != cudaSuccess) return -1;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * sms * 2) != cudaSuccess) return -2;
  const int block = 1024, grid = sms * 2;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  dfma_chains<<<grid, block>>>(out, 16, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  dfma_chains<<<grid, block>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return -3;
  const double fmas = (double)grid * block * iters * 16.0 * 8.0;
  *tflops = 2.0 * fmas / (ms * 1e-3) / 1e12;
  *ms_out = ms;
  return 0;
}
