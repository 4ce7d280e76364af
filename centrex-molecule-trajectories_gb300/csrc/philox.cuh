// Counter-based random numbers for on-device initial conditions.
//
// Philox-4x32-10 as published by Salmon, Moraes, Dror and Shaw, "Parallel
// random numbers: as easy as 1, 2, 3" (SC'11): ten rounds of two 32x32->64
// multiplies with the paper's multipliers and Weyl key increments.  Molecule i
// of a run with (seed, offset) uses key = seed and counter
// (lo32(offset + i), hi32(offset + i), call, 0), so any molecule can be
// regenerated from its index alone (used by the trajectory replay and by
// chunked or multi-replica runs with disjoint offsets).
//
// Uniforms: each 32-bit word w gives U = (w + 1/2) * 2^-32 in (0, 1); the FP32
// path rounds that value to float, so both precisions see the same draws.
// Normals: Box and Muller (1958), sqrt(-2 ln U1) * (cos 2 pi U2, sin 2 pi U2).
// FP64 evaluates them with CUDA's log / log1p, sqrt and sincospi; FP32 with
// the branch-free forms below (log1p from the atanh series, the square root
// as t rsqrt(t), sin and cos of pi a from their Taylor series), within a few
// ulp of the exact values (checked against FP64 on the device by
// bench_kernels/box_muller_check.cu).
#pragma once
#include <cstdint>

namespace ctraj {

struct Philox4 {
  uint32_t v[4];
};

__host__ __device__ inline void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                             uint32_t k0, uint32_t k1) {
  const uint64_t p0 = uint64_t(0xD2511F53u) * c0;
  const uint64_t p1 = uint64_t(0xCD9E8D57u) * c2;
  const uint32_t hi0 = uint32_t(p0 >> 32), lo0 = uint32_t(p0);
  const uint32_t hi1 = uint32_t(p1 >> 32), lo1 = uint32_t(p1);
  const uint32_t n0 = hi1 ^ c1 ^ k0;
  const uint32_t n2 = hi0 ^ c3 ^ k1;
  c0 = n0;
  c1 = lo1;
  c2 = n2;
  c3 = lo0;
}

// The ten round keys of a seed (the key plus r Weyl increments), computed on
// the host once per launch and read from the kernel parameters, so that no
// thread repeats the key schedule.
struct PhiloxKey {
  uint32_t k[20];  // round r: k[2r], k[2r + 1]
};

inline PhiloxKey philox_key(uint64_t seed) {
  PhiloxKey K;
  uint32_t k0 = uint32_t(seed), k1 = uint32_t(seed >> 32);
  for (int r = 0; r < 10; ++r) {
    K.k[2 * r] = k0;
    K.k[2 * r + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return K;
}

__host__ __device__ inline Philox4 philox4x32_10(uint64_t ctr, uint32_t call, const PhiloxKey& K) {
  uint32_t c0 = uint32_t(ctr), c1 = uint32_t(ctr >> 32), c2 = call, c3 = 0u;
#pragma unroll
  for (int r = 0; r < 10; ++r) philox_round(c0, c1, c2, c3, K.k[2 * r], K.k[2 * r + 1]);
  return Philox4{{c0, c1, c2, c3}};
}

// log(1 + x) for x in [-1/2, 1], branch-free: 2 atanh(s) with s = x / (2 + x)
// in [-1/3, 1/3], from the series 2 s (1 + s^2/3 + s^4/5 + ... + s^14/15),
// whose next term is below 1.4e-9 relative; s by the fast division (2 ulp).
__device__ __forceinline__ float log1p_atanh(float x) {
  const float s = __fdividef(x, __fadd_rn(2.0f, x));
  const float s2 = __fmul_rn(s, s);
  float p = 1.0f / 15.0f;
  p = __fmaf_rn(p, s2, 1.0f / 13.0f);
  p = __fmaf_rn(p, s2, 1.0f / 11.0f);
  p = __fmaf_rn(p, s2, 1.0f / 9.0f);
  p = __fmaf_rn(p, s2, 1.0f / 7.0f);
  p = __fmaf_rn(p, s2, 1.0f / 5.0f);
  p = __fmaf_rn(p, s2, 1.0f / 3.0f);
  p = __fmaf_rn(p, s2, 1.0f);
  return __fmul_rn(__fmul_rn(2.0f, s), p);
}

// sin(pi a) and cos(pi a) for a in [0, 2], branch-free: a = j/2 + f with
// j = rint(2a) and |f| <= 1/4 (f exact), x = pi f, the Taylor series of sin
// to x^9 and of cos to x^10 (next terms below 3e-9 and 2e-10 relative for
// |x| <= pi/4), rotated by the quadrant j: sin(j pi/2 + x), cos(j pi/2 + x).
__device__ __forceinline__ void sincospi_taylor(float a, float& sn, float& cs) {
  const float j = rintf(__fmul_rn(2.0f, a));
  const float x = __fmul_rn(__fmaf_rn(-0.5f, j, a), 3.14159265358979323846f);
  const float x2 = __fmul_rn(x, x);
  float ps = 1.0f / 362880.0f;
  ps = __fmaf_rn(ps, x2, -1.0f / 5040.0f);
  ps = __fmaf_rn(ps, x2, 1.0f / 120.0f);
  ps = __fmaf_rn(ps, x2, -1.0f / 6.0f);
  const float s = __fmaf_rn(__fmul_rn(ps, x2), x, x);
  float pc = -1.0f / 3628800.0f;
  pc = __fmaf_rn(pc, x2, 1.0f / 40320.0f);
  pc = __fmaf_rn(pc, x2, -1.0f / 720.0f);
  pc = __fmaf_rn(pc, x2, 1.0f / 24.0f);
  pc = __fmaf_rn(pc, x2, -0.5f);
  const float c = __fmaf_rn(pc, x2, 1.0f);
  const int q = int(j) & 3;
  const float s1 = (q & 1) ? c : s, c1 = (q & 1) ? s : c;
  sn = (q & 2) ? -s1 : s1;
  cs = ((q + 1) & 2) ? -c1 : c1;
}

__device__ __forceinline__ float u01f(uint32_t w) {
  // (w + 1/2) 2^-32 rounded once to float; never 0
  return __fmaf_rn(__uint2float_rn(w), 2.3283064365386963e-10f, 1.1641532182693481e-10f);
}

__device__ __forceinline__ double u01d(uint32_t w) {
  return __fma_rn(double(w), 2.3283064365386963e-10, 1.1641532182693481e-10);
}

// ln U for U = (w + 1/2) 2^-32.  Above one half, U is close to 1 and a float
// holds it only to 2^-25 absolute, which would make the Box-Muller radius
// sqrt(-2 ln U) inaccurate near zero; there ln U = log1p(-V) with
// V = 1 - U = (~w + 1/2) 2^-32 formed exactly from the integer.  Below one
// half, U = 2^e m with m in [1, 2) and ln U = e ln 2 + log1p(m - 1) (m - 1
// exact), so both halves take the same single log1p and no lane diverges.
__device__ __forceinline__ float log_u01f(uint32_t w) {
  const bool low = w < 0x80000000u;
  const float u = u01f(low ? w : ~w);  // U, or V = 1 - U
  const uint32_t bits = __float_as_uint(u);
  const float e = float(int(bits >> 23) - 127);
  const float m1 = __fadd_rn(__uint_as_float((bits & 0x007fffffu) | 0x3f800000u), -1.0f);
  const float l = log1p_atanh(low ? m1 : -u);
  return low ? __fmaf_rn(e, 0.693147180559945309f, l) : l;
}

__device__ __forceinline__ double log_u01d(uint32_t w) {
  return (w < 0x80000000u) ? log(u01d(w)) : log1p(-u01d(~w));
}

__device__ __forceinline__ void box_muller(uint32_t w1, uint32_t w2, float& a, float& b) {
  const float t = __fmul_rn(-2.0f, log_u01f(w1));  // > 0: ln U < 0 for every word
  const float r = __fmul_rn(t, rsqrtf(t));
  float s, c;
  sincospi_taylor(__fmul_rn(2.0f, u01f(w2)), s, c);
  a = __fmul_rn(r, c);
  b = __fmul_rn(r, s);
}

__device__ __forceinline__ void box_muller(uint32_t w1, uint32_t w2, double& a, double& b) {
  const double r = sqrt(__dmul_rn(-2.0, log_u01d(w1)));
  double s, c;
  sincospi(__dmul_rn(2.0, u01d(w2)), &s, &c);
  a = __dmul_rn(r, c);
  b = __dmul_rn(r, s);
}

// The eight words of two Philox calls and how they are used:
//   (w0, w1) -> normals n0, n1 -> vx, vy
//   (w2, w3) -> normals n2, n3 -> vz, Gaussian x
//   (w4, w5) -> normals n4, _  -> Gaussian y
//   w6, w7   -> disc angle and radius (CeNTREXPositionDistribution)
struct Words8 {
  uint32_t w[8];
};

__device__ __forceinline__ Words8 molecule_words(uint64_t id, const PhiloxKey& K) {
  const Philox4 a = philox4x32_10(id, 0u, K);
  const Philox4 b = philox4x32_10(id, 1u, K);
  return Words8{{a.v[0], a.v[1], a.v[2], a.v[3], b.v[0], b.v[1], b.v[2], b.v[3]}};
}

}  // namespace ctraj
