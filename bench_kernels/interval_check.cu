// Part of libctraj_probes.so (bench_kernels/).  Check of the FP32 table-interval computation of the soft-transmission
// kernels and the linear-table lens lookups (table_interval in molecule.cuh) against the truncating float-to-unsigned
// conversion and its inverse it replaces, over generated arguments: random
// bit patterns (negative, NaN, infinite, subnormal and huge values), quarter
// steps across the table and the neighbours of every integer; the form for
// non-negative arguments (table_interval<true>) on those >= 0.
#include <cuda_runtime.h>

#include "molecule.cuh"

namespace {

__device__ __forceinline__ unsigned mix(unsigned x) {
  x ^= x >> 16;
  x *= 0x7feb352du;
  x ^= x >> 15;
  x *= 0x846ca68bu;
  x ^= x >> 16;
  return x;
}

__global__ void k_interval_check(const long long n, const unsigned last, unsigned long long* mismatches) {
  unsigned long long bad = 0;
  const float last_f = __uint2float_rn(last);
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    float s;
    const unsigned kk = unsigned(k);
    switch (kk % 4u) {
      case 0: s = __uint_as_float(mix(kk)); break;                                    // any bit pattern
      case 1: s = __fmul_rn(__int2float_rn(int(kk / 4u % 40000u) - 8000), 0.25f); break;  // quarter steps
      case 2: s = __uint_as_float(__float_as_uint(__int2float_rn(int(kk / 4u % 9000u))) - 1u); break;  // below an integer
      default: s = __uint_as_float(__float_as_uint(__int2float_rn(int(kk / 4u % 9000u))) + 1u); break;  // above
    }
    unsigned i;
    float u;
    ctraj::table_interval(s, last, last_f, i, u);
    const unsigned i_ref = min(__float2uint_rz(s), last);
    const float u_ref = __fadd_rn(s, -__uint2float_rn(i_ref));
    const bool same_u = __float_as_uint(u) == __float_as_uint(u_ref) || (isnan(u) && isnan(u_ref));
    bad += (i != i_ref || !same_u) ? 1 : 0;
    if (s >= 0.0f) {  // the form without max(s, 0), on the arguments it is given
      unsigned i2;
      float u2;
      ctraj::table_interval<true>(s, last, last_f, i2, u2);
      bad += (i2 != i_ref || __float_as_uint(u2) != __float_as_uint(u_ref)) ? 1 : 0;
    }
  }
  if (bad) atomicAdd(mismatches, bad);
}

}  // namespace

// Returns 0 and the number of arguments (of n) where the two computations
// differ, for the clamp `last` (the table's last interval index).
extern "C" int ctraj_peak_interval_check(long long n, unsigned last, unsigned long long* mismatches) {
  if (n < 1 || !mismatches) return -1;
  unsigned long long* d = nullptr;
  if (cudaMalloc(&d, sizeof *d) != cudaSuccess) return -3;
  cudaMemset(d, 0, sizeof *d);
  k_interval_check<<<1024, 256>>>(n, last, d);
  cudaError_t e = cudaMemcpy(mismatches, d, sizeof *d, cudaMemcpyDeviceToHost);
  cudaFree(d);
  return e == cudaSuccess ? 0 : -2;
}
