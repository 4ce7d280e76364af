// libctraj_probes.so (bench_kernels/): measures the FP32 FMA throughput of the current GPU, the
// denominator of the lens kernel's roofline fraction (the lens RK4 is bound by
// the FP32 CUDA-core pipe, not by HBM or tensor cores).
//
// Each thread runs 8 independent FMA chains; the grid fills every SM with 8
// resident 256-thread blocks.  FLOPs = 2 per FMA.  Timed with CUDA events on
// a private stream after one warm-up launch.
#include <cuda_runtime.h>

namespace {

__global__ void __launch_bounds__(256) k_fma(float* out, int iters) {
  float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-3f, a2 = a0 + 2e-3f, a3 = a0 + 3e-3f;
  float a4 = a0 + 4e-3f, a5 = a0 + 5e-3f, a6 = a0 + 6e-3f, a7 = a0 + 7e-3f;
  const float b = 0.9999f, c = 1e-4f;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      a0 = __fmaf_rn(a0, b, c); a1 = __fmaf_rn(a1, b, c); a2 = __fmaf_rn(a2, b, c); a3 = __fmaf_rn(a3, b, c);
      a4 = __fmaf_rn(a4, b, c); a5 = __fmaf_rn(a5, b, c); a6 = __fmaf_rn(a6, b, c); a7 = __fmaf_rn(a7, b, c);
    }
  }
  const float s = ((a0 + a1) + (a2 + a3)) + ((a4 + a5) + (a6 + a7));
  if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live; never true
}

}  // namespace

extern "C" int ctraj_peak_fp32(int device, int iters, double* tflops, double* ms) {
  if (cudaSetDevice(device) != cudaSuccess) return -2;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256;
  float* out = nullptr;
  cudaStream_t s;
  cudaEvent_t e0, e1;
  if (cudaMalloc(&out, blocks * sizeof(float)) != cudaSuccess) return -3;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma<<<blocks, threads, 0, s>>>(out, iters / 10 + 1);
  cudaEventRecord(e0, s);
  k_fma<<<blocks, threads, 0, s>>>(out, iters);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaEventSynchronize(e1);
  float t = 0.f;
  cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(out);
  if (err != cudaSuccess) return -2;
  const double flops = 2.0 * 8.0 * 16.0 * double(iters) * double(blocks) * threads;
  *ms = t;
  *tflops = flops / (double(t) * 1e-3) / 1e12;
  return 0;
}
