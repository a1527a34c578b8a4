// xg_smem.cuh — a kernel's dynamic shared-memory limit, only ever raised.
#pragma once

#include <cuda_runtime.h>

#include <map>
#include <mutex>
#include <utility>

namespace xg {

// The dynamic shared memory a kernel may take is one setting per kernel and
// device for the whole process.  Objects set up with different sizes share
// it (slotted batches of other size classes, factorisations of other
// matrices), and one set up later must not lower it under the launches of
// another: it only grows.  cudaSuccess when `bytes` are allowed.
inline cudaError_t allow_dynamic_smem(const void *kernel, size_t bytes) {
  static std::mutex m;
  static std::map<std::pair<int, const void *>, size_t> granted;
  int dev = 0;
  cudaGetDevice(&dev);
  std::lock_guard<std::mutex> lock(m);
  size_t &g = granted[{dev, kernel}];
  if (bytes <= g) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return e;
  }
  g = bytes;
  return cudaSuccess;
}

}  // namespace xg
