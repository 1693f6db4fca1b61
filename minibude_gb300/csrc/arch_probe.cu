// arch_probe.cu -- the architecture check behind bude_gpu_compatible; replaces the reference's
// `version` kernel and CudaBude::compatible (src/cuda/fasten.hpp:12-18, 218-248).
#include <cuda_runtime.h>

#include "internal.h"

namespace bude {

__global__ void arch_probe_kernel(int *out) {
#ifdef __CUDA_ARCH__
  out[0] = __CUDA_ARCH__ / 10; // e.g. 1030 -> 103
#else
  out[0] = -1;
#endif
}

int probe_kernel_arch(int device, int *cc) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  int *d = nullptr;
  e = cudaMalloc(&d, sizeof(int));
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
  int h = -2;
  arch_probe_kernel<<<1, 1>>>(d);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&h, d, sizeof(int), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return cuda_error(e, "architecture probe kernel");
  *cc = h;
  return BUDE_OK;
}

} // namespace bude
