// Part of libctraj_probes.so (bench_kernels/).  Accuracy of the FP32 Box-Muller
// transform of the on-device initial conditions (philox.cuh: log1p_atanh,
// sincospi_taylor, box_muller<float>) against the FP64 transform of the same
// words, and of CUDA's own FP32 functions (log1pf, sqrtf, sincospif) on the
// same arguments for comparison.  Arguments: hashed words, every word near
// 0, 2^31 and 2^32 - 1 (the ends of both halves of log U), and even steps of
// x in [-1/2, 1] and of a in [0, 2].
#include <cuda_runtime.h>

#include "philox.cuh"

namespace {

__device__ __forceinline__ unsigned mix(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

// the FP32 transform with CUDA's functions, for the comparison column
__device__ __forceinline__ float log_u01f_libm(uint32_t w) {
  const bool low = w < 0x80000000u;
  const float u = ctraj::u01f(low ? w : ~w);
  const uint32_t bits = __float_as_uint(u);
  const float e = float(int(bits >> 23) - 127);
  const float m1 = __fadd_rn(__uint_as_float((bits & 0x007fffffu) | 0x3f800000u), -1.0f);
  const float l = log1pf(low ? m1 : -u);
  return low ? __fmaf_rn(e, 0.693147180559945309f, l) : l;
}

__device__ __forceinline__ void box_muller_libm(uint32_t w1, uint32_t w2, float& a, float& b) {
  const float r = sqrtf(__fmul_rn(-2.0f, log_u01f_libm(w1)));
  float s, c;
  sincospif(__fmul_rn(2.0f, ctraj::u01f(w2)), &s, &c);
  a = __fmul_rn(r, c);
  b = __fmul_rn(r, s);
}

__device__ __forceinline__ void atomic_max_pos(float* p, float v) {
  if (v > 0.0f) atomicMax(reinterpret_cast<int*>(p), __float_as_int(v));  // non-negative floats order as ints
}

// out[0]: largest |normal - FP64 normal| / FP64 radius (this transform)
// out[1]: the same for CUDA's FP32 functions
// out[2]: largest relative error of log1p_atanh on [-1/2, 1]
// out[3]: the same for log1pf
// out[4]: largest absolute error of sincospi_taylor on [0, 2]
// out[5]: the same for sincospif
__global__ void k_bm_check(const long long n, float* out) {
  float e[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const unsigned kk = unsigned(k);
    unsigned w1 = mix(kk), w2 = mix(kk ^ 0x9e3779b9u);
    switch (kk % 8u) {
      case 1: w1 = kk / 8u % 65536u; break;                 // U near 0
      case 2: w1 = 0x80000000u + (kk / 8u % 65536u) - 32768u; break;  // the two halves meet
      case 3: w1 = 0xFFFFFFFFu - (kk / 8u % 65536u); break;  // U near 1: the radius near 0
      default: break;
    }
    float a, b, al, bl;
    double ad, bd;
    ctraj::box_muller(w1, w2, a, b);
    box_muller_libm(w1, w2, al, bl);
    ctraj::box_muller(w1, w2, ad, bd);
    const double r = sqrt(ad * ad + bd * bd);
    if (r > 0.0) {
      e[0] = fmaxf(e[0], float(fmax(fabs(double(a) - ad), fabs(double(b) - bd)) / r));
      e[1] = fmaxf(e[1], float(fmax(fabs(double(al) - ad), fabs(double(bl) - bd)) / r));
    }
    const float x = __fmaf_rn(float(kk % 3000001u), 5.0e-7f, -0.5f);  // [-1/2, 1]
    const double l = log1p(double(x));
    if (l != 0.0) {
      e[2] = fmaxf(e[2], float(fabs(double(ctraj::log1p_atanh(x)) - l) / fabs(l)));
      e[3] = fmaxf(e[3], float(fabs(double(log1pf(x)) - l) / fabs(l)));
    }
    const float t = __fmul_rn(float(kk % 4000001u), 5.0e-7f);  // [0, 2]
    double sd, cd;
    sincospi(double(t), &sd, &cd);
    float st, ct, sl, cl;
    ctraj::sincospi_taylor(t, st, ct);
    sincospif(t, &sl, &cl);
    e[4] = fmaxf(e[4], float(fmax(fabs(double(st) - sd), fabs(double(ct) - cd))));
    e[5] = fmaxf(e[5], float(fmax(fabs(double(sl) - sd), fabs(double(cl) - cd))));
  }
  for (int j = 0; j < 6; ++j) atomic_max_pos(out + j, e[j]);
}

}  // namespace

// Returns 0 and the six largest errors above (out[6]) over n arguments.
extern "C" int ctraj_peak_bm_check(long long n, float* out) {
  if (n < 1 || !out) return -1;
  float* d = nullptr;
  if (cudaMalloc(&d, 6 * sizeof(float)) != cudaSuccess) return -3;
  cudaMemset(d, 0, 6 * sizeof(float));
  k_bm_check<<<1024, 256>>>(n, d);
  cudaError_t e = cudaMemcpy(out, d, 6 * sizeof(float), cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : -2;
}
