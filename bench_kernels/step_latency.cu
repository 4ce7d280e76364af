// Part of libctraj_probes.so (bench_kernels/): the production FP32 lens RK4 step
// (Mol32::lens_step with the table staged in shared memory) run in a loop on
// a fixed set of molecules, timed with clock64 and CUDA events.
//
// With one warp it measures the step's latency (cycles per step), the floor
// for a molecule that is alone on its SM.  With 2 CTAs of 512 threads per SM
// it measures the step's throughput (lane-steps per second) without the
// queue, compaction and early-loss effects of a real run.
#include <cuda_runtime.h>

#include "molecule.cuh"

namespace {

using ctraj::LensArgs;

template <int F>
__global__ void __launch_bounds__(512) k_step_loop(LensArgs L, int steps, float dt, long long* cyc,
                                                   float* out) {
  extern __shared__ float4 s_tab[];
  for (int k = threadIdx.x; k < L.n_int; k += blockDim.x) s_tab[k] = L.q[k];
  __syncthreads();
  ctraj::Mol32<false, false> m;
  // a spread of near-axis molecules, as in the long-lived tail of a run
  m.x = 2e-3f * (1.0f + 1e-3f * float(threadIdx.x));
  m.y = 1e-3f;
  m.vx = 0.5f;
  m.vy = -0.3f;
  m.cx = m.cy = m.cvx = m.cvy = 0.0f;
  m.ax = 0.0f;
  m.ay = -L.g;
  const float hdt = 0.5f * dt, dt6 = dt * (1.0f / 6.0f), dt26 = dt * dt * (1.0f / 6.0f);
  unsigned flags = 0;
  int lost = 0;
  const long long t0 = clock64();
  for (int n = 0; n < steps; ++n)
    lost += m.template lens_step<F, true>(L, dt, hdt, dt, dt6, dt26, s_tab, flags);
  const long long t1 = clock64();
  if (threadIdx.x == 0) cyc[blockIdx.x] = t1 - t0;
  out[blockIdx.x * blockDim.x + threadIdx.x] = m.x + m.y + m.vx + m.vy + float(lost + int(flags));
}

}  // namespace

// q: FP32 Stark table in device memory, in one of the lens kernels' layouts:
// linear = 1: n_int float4 of two (w, dw) quarter-interval pieces, beta in
// quarter intervals (kForceStark2Lin); linear = 0: one (a, b, c, 0) quadratic
// per interval (kForceStark2).
// Returns 0 and the mean clock64 cycles per step and lane-steps per second.
extern "C" int ctraj_peak_step(const void* q, int n_int, float beta, int linear, int steps, int blocks,
                               int threads, double* cycles_per_step, double* lane_steps_per_s) {
  if (!q || n_int < 1 || n_int > 8192 || steps < 1 || blocks < 1 || threads < 32 || threads > 512) return -1;
  auto kernel = linear ? k_step_loop<ctraj::kForceStark2Lin> : k_step_loop<ctraj::kForceStark2>;
  LensArgs L{};
  L.q = static_cast<const float4*>(q);
  L.beta = beta;
  L.s0 = 0.0f;
  L.r_max = INFINITY;
  L.n_int = n_int;
  L.n_smem = n_int;
  L.g = 9.80665f;
  L.bore2 = 1.0f;
  L.bore = 1.0f;
  long long* cyc = nullptr;
  float* out = nullptr;
  if (cudaMalloc(&cyc, blocks * sizeof(long long)) != cudaSuccess) return -3;
  if (cudaMalloc(&out, size_t(blocks) * threads * sizeof(float)) != cudaSuccess) {
    cudaFree(cyc);
    return -3;
  }
  const size_t smem = size_t(n_int) * sizeof(float4);
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem));
  cudaStream_t s;
  cudaEvent_t e0, e1;
  cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  kernel<<<blocks, threads, smem, s>>>(L, 32, 1e-6f, cyc, out);
  cudaEventRecord(e0, s);
  kernel<<<blocks, threads, smem, s>>>(L, steps, 1e-6f, cyc, out);
  cudaEventRecord(e1, s);
  cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  long long* h = new long long[blocks];
  cudaMemcpy(h, cyc, blocks * sizeof(long long), cudaMemcpyDeviceToHost);
  double mean = 0.0;
  for (int b = 0; b < blocks; ++b) mean += double(h[b]);
  delete[] h;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  cudaFree(cyc);
  cudaFree(out);
  if (err != cudaSuccess) return -2;
  *cycles_per_step = mean / blocks / steps;
  *lane_steps_per_s = double(blocks) * threads * steps / (double(ms) * 1e-3);
  return 0;
}
