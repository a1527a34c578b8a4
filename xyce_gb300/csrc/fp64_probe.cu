// fp64_probe.cu — measures this GPU's sustained FP64 fused multiply-add rate:
// the roofline denominator for the device-evaluation kernels, which are
// bound by the FP64 pipe (GB300 issues two FP64 thread operations per cycle
// per SM).  Eight independent DFMA chains per thread, one block per SM slot,
// timed with CUDA events.

#include <cuda_runtime.h>

#include "xg.h"
#include "xg_fast_rcp.cuh"
#include "xg_internal.h"

namespace {

__global__ void __launch_bounds__(256) dfma_chains(double *out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-3, x2 = x0 + 2e-3, x3 = x0 + 3e-3;
  double x4 = x0 + 4e-3, x5 = x0 + 5e-3, x6 = x0 + 6e-3, x7 = x0 + 7e-3;
  for (int k = 0; k < iters; ++k) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 1234.5678) out[blockIdx.x] = s;  // keeps the chains live
}

__global__ void reciprocals(const double *b, double *out, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = xg::fast_rcp(b[i]);
}

}  // namespace

extern "C" int xg_probe_reciprocal(int n, const double *host_b, double *host_out) {
  if (n < 0 || (n && (!host_b || !host_out))) return XG_ERR_ARG;
  if (!n) return XG_OK;
  double *d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * 2 * size_t(n)) != cudaSuccess) return XG_ERR_OOM;
  cudaError_t e = cudaMemcpy(d, host_b, sizeof(double) * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    reciprocals<<<(n + 255) / 256, 256>>>(d, d + n, n);
    xg::count_launches(1);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(host_out, d + n, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

extern "C" int xg_probe_fp64_rate(int cuda_device, double *flops_per_second) {
  if (!flops_per_second) return XG_ERR_ARG;
  if (cudaSetDevice(cuda_device) != cudaSuccess) return XG_ERR_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, cuda_device) != cudaSuccess)
    return XG_ERR_CUDA;
  const int blocks = sms * 8, threads = 256, iters = 4096;
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return XG_ERR_CUDA;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const double a = 0.999999, b = 1e-7;
  dfma_chains<<<blocks, threads, 0, s>>>(nullptr, 64, a, b);  // warm-up
  float best_ms = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0, s);
    dfma_chains<<<blocks, threads, 0, s>>>(nullptr, iters, a, b);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) best_ms = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (err != cudaSuccess) return XG_ERR_CUDA;
  const double flops = 2.0 * 8.0 * (double)iters * blocks * threads;
  *flops_per_second = flops / (best_ms * 1e-3);
  return XG_OK;
}
