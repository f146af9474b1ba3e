// ecp_peaks.cu -- pipe-throughput probe (FP64 FMA, FP32 FMA, MUFU ex2, FP64
// exp) on the current device.  The ECP kernels are bound by these pipes, not
// by HBM, so their roofline denominators are measured here: the same code,
// same clocks, same box as the timed run.
#include <cuda_runtime.h>

#include "ecp_host.h"

namespace ecpgb {

template <typename T>
__global__ void k_fma(T *out, int iters, T a, T b) {
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
    x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      x0 = x0 * a + b; x1 = x1 * a + b; x2 = x2 * a + b; x3 = x3 * a + b;
      x4 = x4 * a + b; x5 = x5 * a + b; x6 = x6 * a + b; x7 = x7 * a + b;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

__global__ void k_ex2(float *out, int iters) {
  float x0 = threadIdx.x * 1e-3f, x1 = x0 + 0.1f, x2 = x0 + 0.2f, x3 = x0 + 0.3f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x0));
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x1));
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x2));
      asm volatile("ex2.approx.ftz.f32 %0, %0;" : "+f"(x3));
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

__global__ void k_dexp(double *out, int iters) {
  double x0 = -(threadIdx.x % 7) * 0.37, x1 = x0 - 0.1, x2 = x0 - 0.2, x3 = x0 - 0.3, s = 0;
  for (int i = 0; i < iters; i++) {
#pragma unroll 4
    for (int k = 0; k < 16; k++) {
      s += exp(x0) + exp(x1) + exp(x2) + exp(x3);
      x0 -= 1e-6; x1 -= 1e-6; x2 -= 1e-6; x3 -= 1e-6;
    }
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

int measure_peaks(double *out) {
  int dev = 0;
  cudaDeviceProp p;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&p, dev) != cudaSuccess) {
    set_error("no CUDA device");
    return 1;
  }
  const int threads = 256, blocks = p.multiProcessorCount * 8;
  void *buf = nullptr;
  if (cudaMalloc(&buf, (size_t)blocks * threads * 8) != cudaSuccess) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float ms;
  double nthr = (double)blocks * threads;
  auto timed = [&](auto launch) {
    launch(2);
    cudaDeviceSynchronize();
    cudaEventRecord(e0);
    launch(0);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    return (double)ms;
  };
  int it = 1000;
  double t = timed([&](int w) { k_fma<double><<<blocks, threads>>>((double *)buf, w ? w : it, 1.0000001, 1e-9); });
  out[0] = 2.0 * nthr * it * 128 / (t * 1e9);
  it = 20000;
  t = timed([&](int w) { k_fma<float><<<blocks, threads>>>((float *)buf, w ? w : it, 1.0000001f, 1e-9f); });
  out[1] = 2.0 * nthr * it * 128 / (t * 1e9);
  it = 5000;
  t = timed([&](int w) { k_ex2<<<blocks, threads>>>((float *)buf, w ? w : it); });
  out[2] = nthr * it * 64 / (t * 1e6);
  it = 100;
  t = timed([&](int w) { k_dexp<<<blocks, threads>>>((double *)buf, w ? w : it); });
  out[3] = nthr * it * 64 / (t * 1e6);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(buf);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

}  // namespace ecpgb
