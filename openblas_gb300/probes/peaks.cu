// Peak-rate probes for the roofline denominators the driver does not
// measure: the FP64 rate of one GB300 as DFMA (scalar fused multiply-add)
// and as DMMA (mma.sync m8n8k4 f64), and the tcgen05 kind::f16 (bf16) MMA
// issue rate of this build's own kernels.  Each probe times one launch of a
// kernel whose work is independent chains of the instruction under test,
// with CUDA events, after one warm-up launch.  This library is measurement
// infrastructure (bench.py --peaks); the BLAS library does not use it.
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int CHAINS = 16;

// A 4 x 4 outer-product update per iteration, as in a register-tiled GEMM:
// CHAINS = 16 independent accumulators c_ij <- a_i * b_j + c_ij.
__global__ void __launch_bounds__(256) dfma_kernel(int iters, double x, double y, double *out) {
  double a[4], b[4], c[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    a[i] = x + threadIdx.x + i;
    b[i] = y - i;
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) c[i][j] = 0.0;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 4; ++j) c[i][j] = fma(a[i], b[j], c[i][j]);
  }
  double s = 0.0;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) s += c[i][j];
  if (s == 12345.678) out[0] = s;  // keeps the chains live
}

// Four independent m8n8k4 FP64 MMA accumulators per warp.
__global__ void __launch_bounds__(256) dmma_kernel(int iters, double x, double *out) {
  double a = x + threadIdx.x, b = x - threadIdx.x;
  double d[4][2];
#pragma unroll
  for (int c = 0; c < 4; ++c) d[c][0] = d[c][1] = 0.0;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
          : "+d"(d[c][0]), "+d"(d[c][1])
          : "d"(a), "d"(b));
  }
  double s = 0.0;
#pragma unroll
  for (int c = 0; c < 4; ++c) s += d[c][0] + d[c][1];
  if (s == 12345.678) out[0] = s;
}

template <typename K>
int time_kernel(K launch, double flops, double *tflops) {
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return 2;
  launch();  // warm-up
  cudaEventRecord(e0);
  launch();
  cudaEventRecord(e1);
  cudaError_t e = cudaEventSynchronize(e1);
  float ms = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess || ms <= 0.f) return 2;
  *tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 0;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 0;
  return n;
}

}  // namespace

extern "C" {

// DFMA rate over all SMs (4 CTAs of 256 threads per SM, 16 independent
// accumulators per thread).  Returns 0 on success.
int gbp_fp64_dfma_tflops(double *tflops) {
  const int sms = sm_count();
  if (sms <= 0) return 1;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return 2;
  const int iters = 1 << 13, blocks = sms * 4, threads = 256;
  const double flops = 2.0 * CHAINS * (double)iters * blocks * threads;
  const int st = time_kernel(
      [&] { dfma_kernel<<<blocks, threads>>>(iters, 0.5, 0.25, out); }, flops, tflops);
  cudaFree(out);
  return st ? st : (cudaGetLastError() == cudaSuccess ? 0 : 2);
}

// DMMA (mma.sync m8n8k4 f64) rate over all SMs: 512 flops per warp MMA.
int gbp_fp64_dmma_tflops(double *tflops) {
  const int sms = sm_count();
  if (sms <= 0) return 1;
  double *out = nullptr;
  if (cudaMalloc(&out, sizeof(double)) != cudaSuccess) return 2;
  const int iters = 1 << 13, blocks = sms * 4, threads = 256;
  const double flops = 512.0 * 4 * (double)iters * blocks * (threads / 32);
  const int st =
      time_kernel([&] { dmma_kernel<<<blocks, threads>>>(iters, 0.5, out); }, flops, tflops);
  cudaFree(out);
  return st ? st : (cudaGetLastError() == cudaSuccess ? 0 : 2);
}

}  // extern "C"
