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
// Normals: Box and Muller (1958), sqrt(-2 ln U1) * (cos 2 pi U2, sin 2 pi U2),
// evaluated with CUDA's own logf/log, sqrtf/sqrt and sincospif/sincospi.
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
// exact), so both halves take the same single log1pf and no lane diverges.
__device__ __forceinline__ float log_u01f(uint32_t w) {
  const bool low = w < 0x80000000u;
  const float u = u01f(low ? w : ~w);  // U, or V = 1 - U
  const uint32_t bits = __float_as_uint(u);
  const float e = float(int(bits >> 23) - 127);
  const float m1 = __fadd_rn(__uint_as_float((bits & 0x007fffffu) | 0x3f800000u), -1.0f);
  const float l = log1pf(low ? m1 : -u);
  return low ? __fmaf_rn(e, 0.693147180559945309f, l) : l;
}

__device__ __forceinline__ double log_u01d(uint32_t w) {
  return (w < 0x80000000u) ? log(u01d(w)) : log1p(-u01d(~w));
}

__device__ __forceinline__ void box_muller(uint32_t w1, uint32_t w2, float& a, float& b) {
  const float r = sqrtf(__fmul_rn(-2.0f, log_u01f(w1)));
  float s, c;
  sincospif(__fmul_rn(2.0f, u01f(w2)), &s, &c);
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
