// L2 read-bandwidth probe: the denominator the benchmark reports the step
// kernel's achieved bytes against when its working set lives in L2.
//
// One buffer of `bytes` (small enough to stay in the 129 MB L2) is read once
// to bring it into L2, then `reps` times over by one kernel with 16-byte
// loads that bypass L1 (ld.global.cg), every SM reading the whole buffer in
// a grid-stride order; CUDA events time the kernel, best of five launches.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/sop_gpu.h"

namespace {

__global__ void __launch_bounds__(512) k_l2_read(const float4* __restrict__ p, long long n4, int reps,
                                                 float* sink) {
  float ax = 0.f, ay = 0.f, az = 0.f, aw = 0.f;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (int r = 0; r < reps; r++) {
    // each repetition starts at another offset, so an SM's slice changes
    const long long shift = ((long long)r * (stride / 7 + 1)) % n4;  // < n4, so i < 2 n4
    for (long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += stride) {
      long long i = k + shift;
      if (i >= n4) i -= n4;
      const float4 v = __ldcg(p + i);
      ax += v.x; ay += v.y; az += v.z; aw += v.w;
    }
  }
  // the buffer holds zeros, so this never stores; the compiler cannot know
  if (ax + ay + az + aw != 0.f) sink[0] = ax + ay + az + aw;
}

}  // namespace

extern "C" int sop_probe_l2_read(int device, int64_t bytes, int reps, double* gbs) {
  if (!gbs || bytes < (1 << 20) || bytes > ((int64_t)96 << 20) || reps < 1 || reps > 1000)
    return SOP_ERR_ARG;
  *gbs = 0.0;
  if (cudaSetDevice(device) != cudaSuccess) return SOP_ERR_NODEV;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return SOP_ERR_CUDA;
  float4* buf = nullptr;
  float* sink = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  const long long n4 = bytes / 16;
  int rc = SOP_OK;
  float best = 1e30f;
  if (cudaMalloc(&buf, n4 * 16) != cudaSuccess || cudaMalloc(&sink, sizeof(float)) != cudaSuccess ||
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    rc = SOP_ERR_NOMEM;
  } else if (cudaMemsetAsync(buf, 0, n4 * 16, s) != cudaSuccess) {
    rc = SOP_ERR_CUDA;
  } else {
    const int grid = prop.multiProcessorCount * 4;
    k_l2_read<<<grid, 512, 0, s>>>(buf, n4, 1, sink);  // bring the buffer into L2
    for (int t = 0; t < 5 && rc == SOP_OK; t++) {
      cudaEventRecord(e0, s);
      k_l2_read<<<grid, 512, 0, s>>>(buf, n4, reps, sink);
      cudaEventRecord(e1, s);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        rc = SOP_ERR_CUDA;
      else if (ms > 0.f && ms < best)
        best = ms;
    }
    if (rc == SOP_OK && cudaGetLastError() != cudaSuccess) rc = SOP_ERR_CUDA;
  }
  if (rc == SOP_OK && best < 1e30f) *gbs = (double)n4 * 16.0 * reps / (best * 1e-3) / 1e9;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (sink) cudaFree(sink);
  if (buf) cudaFree(buf);
  return rc;
}
