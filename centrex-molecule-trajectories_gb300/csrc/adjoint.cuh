// Soft transmission of the lens beamline and its discrete adjoint.
//
// The soft model replaces every hard aperture test of the propagation
// (CircularAperture at its two planes, apertures.py:101-115, in front of the
// lens and behind it; the lens entrance and the bore test after each RK4
// step, electrostatic_lens.py:60-66, 112-118) by a sigmoid of the edge
// distance: a molecule at radius r in front
// of an edge of radius R keeps the weight sigma((R - r) / w), w the sigmoid
// width, and no molecule is removed.  The soft transmission is the mean over
// molecules of the product of all weights, i.e. exp(sum of log-sigmoids); as
// w -> 0 it becomes the detected fraction.  A molecule whose log weight falls
// below `log_floor` (or is not a number) is dropped: its weight, at most
// exp(log_floor), and its gradient are counted as zero.
//
// Parameters (in this order): lens voltage V, lens z0, the radius of one
// circular aperture (in front of the lens or behind it), the clip radius of
// the lens bore (the field radius stays fixed), and the standard deviations
// of vx and vy.
// Initial conditions are reparameterised: vx = mu_vx + sigma_vx n0 with n0 a
// unit normal from the same Philox draw as ctraj_run (or given by the caller).
//
// Dynamics are the reference's: closed-form ballistic flights with
// a = (0, -g), and inside the lens the fixed-step RK4 of
// electrostatic_lens.py:91-111 (stage-2 point x + dt k1 unless the classic
// scheme is chosen) with step count rint(L/dz) and dt = dz/vz, for the
// hexapole force a_perp = w(r^2) (x, y) - g y^, w = kappa P(s), P the
// derivative W'(E) of the cubic Stark spline on interval i at local
// coordinate u = s - i, s = beta r^2 - s0, beta = alpha / h, kappa =
// -2 alpha / m, alpha = 3 V / R^3.  Behind the lens a molecule flies with
// a = (0, -g) from its state after the last RK4 step, at z0 + N dz, to each
// aperture plane (the reference's exit snap to z1 with the last step's lens
// force, electrostatic_lens.py:74-77, a sub-step of at most dz / 2, is taken
// as part of that ballistic flight: positions differ by nanometres).
//
// Gradients are the exact derivatives of this discrete computation (a
// discrete adjoint): the forward pass stores the lens state every
// `checkpoint` steps; the backward pass recomputes each segment from its
// checkpoint into a per-thread tape (state and force polynomial values at the
// four RK4 stage points) and runs the transposed step Jacobians over it in
// reverse, accumulating dlog(T)/dV; the ballistic part is recomputed and
// reversed the same way, giving d/d(lens z0) from the last flight time and
// d/d(sigma_v) from the initial velocities; the part behind the lens is
// closed form and its adjoint (d/d(state after the lens), d/d(lens z0)) is
// computed in the forward pass and starts the backward composition.  The
// radius derivatives need no adjoint (they do not change the dynamics) and are
// summed in the forward pass.
#pragma once
#include <type_traits>

#include "kernels.cuh"

namespace ctraj {

enum : int {
  kSoftV = 0,
  kSoftZ0 = 1,
  kSoftAperture = 2,
  kSoftBore = 3,
  kSoftSigmaVx = 4,
  kSoftSigmaVy = 5,
  kSoftParams = 6,
};
constexpr int kSoftMaxPlanes = 2 * CTRAJ_MAX_ELEMENTS + 1;
constexpr int kSoftTape = 64;  // largest checkpoint interval (tape entries per thread)
constexpr int kSoftThreads = 128;

// Stat slots of a soft run (unsigned long long).
enum : int { kSoftStatEntered = 0, kSoftStatSteps = 1, kSoftStatDropped = 2, kSoftStatBad = 3, kSoftStatCount = 4 };

// One table interval, padded to one 16-byte (float) or 32-byte (double)
// shared-memory access.
template <class T>
struct alignas(4 * sizeof(T)) Coef4 {
  T q0, q1, q2, pad;
};

// IEEE-rounded arithmetic without contraction, for both precisions, so that
// the checkpoint recomputation repeats the forward pass bit for bit.
__device__ __forceinline__ float add_(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float mul_(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fma_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double add_(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double mul_(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double fma_(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float sqrt_(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double sqrt_(double a) { return __dsqrt_rn(a); }
__device__ __forceinline__ float div_(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rcp_(float a) { return __frcp_rn(a); }
__device__ __forceinline__ double rcp_(double a) { return __drcp_rn(a); }
__device__ __forceinline__ float exp_(float a) { return expf(a); }
__device__ __forceinline__ double exp_(double a) { return exp(a); }
__device__ __forceinline__ float log1p_(float a) { return log1pf(a); }
__device__ __forceinline__ double log1p_(double a) { return log1p(a); }
__device__ __forceinline__ unsigned to_uint_rz(float a) { return __float2uint_rz(a); }
__device__ __forceinline__ unsigned to_uint_rz(double a) { return __double2uint_rz(a); }

// log sigma(z) and sigma(-z) = d log sigma(z) / dz.  With e = exp(-|z|) in
// (0, 1]: log sigma(z) = -log(1 + e) for z >= 0 and z - log(1 + e) below;
// sigma(-z) = e / (1 + e) for z >= 0 and 1 / (1 + e) below.
// FP32 without a branch, so that the lens pass's bore tests interleave with
// its RK4 steps (a branch on z there doubled the step time): log(1 + e) from
// the atanh series (log1p_atanh), 1 / (1 + e) by the fast division (2 ulp).
// FP64: log1p and the IEEE reciprocal.
template <class T>
__device__ __forceinline__ void log_sigmoid(T z, T& ls, T& dls) {
  if constexpr (std::is_same<T, float>::value) {
    const float e = exp_(-fabsf(z));
    const float l = log1p_atanh(e);
    ls = z >= 0.0f ? -l : add_(z, -l);
    dls = mul_(z >= 0.0f ? e : 1.0f, __fdividef(1.0f, add_(1.0f, e)));
  } else {
    const T e = exp_(z >= T(0) ? -z : z);
    const T l = log1p_(e);
    ls = z >= T(0) ? -l : add_(z, -l);
    dls = mul_(z >= T(0) ? e : T(1), rcp_(add_(T(1), e)));
  }
}

// The soft test of an edge of radius R at (x, y): log weight ls and its
// derivative d with respect to R.
// Radius of a soft edge test: FP64 the IEEE square root; FP32 r2 * rsqrt(r2),
// within 2 ulp (the IEEE square root cost a tenth of the soft lens pass).
template <class T>
__device__ __forceinline__ T soft_radius(T x, T y) {
  const T r2 = fma_(y, y, mul_(x, x));
  if constexpr (std::is_same<T, float>::value) {
    return r2 > 0.0f ? mul_(r2, rsqrtf(r2)) : 0.0f;
  } else {
    return sqrt_(r2);
  }
}

template <class T>
__device__ __forceinline__ void soft_test(T x, T y, T R, T inv_w, T& ls, T& d) {
  const T r = soft_radius(x, y);
  T dls;
  log_sigmoid(mul_(add_(R, -r), inv_w), ls, dls);
  d = mul_(dls, inv_w);
}

// Launch-time constants of a soft run.
struct SoftPlan {
  int64_t n;                        // molecules of the whole run
  int64_t first, count;             // the molecules of this launch: first .. first + count - 1
  uint64_t seed, offset;
  PhiloxKey key;                    // round keys of seed
  int ic_mode;
  int n_planes;                     // ballistic planes up to and including the lens entrance
  const double* normals;            // (5, n) unit normals n_vx, n_vy, n_vz, n_x, n_y (host mode)
  double z_ic;                      // initial z
  double sx, sy;                    // position standard deviations
  double mu_vx, mu_vy, mu_vz, s_vz;
  double s_vx, s_vy;                // parameters
  double z[kSoftMaxPlanes];         // plane positions; the last is the lens entrance (lens z0)
  double radius[kSoftMaxPlanes];    // edge radius at the plane; INFINITY: no test
  int param[kSoftMaxPlanes];        // 1: the radius is the aperture parameter
  int n_post;                       // aperture planes behind the lens
  double post_z[kSoftMaxPlanes];
  double post_radius[kSoftMaxPlanes];
  int post_param[kSoftMaxPlanes];
  ctraj_element lens;               // step mode, dz / dt, L (p[7]), scheme; z0 = the parameter
  double V;
  double s0, beta, kappa, kappa1;   // table coordinate and force scales (kappa1 = kappa / V)
  double bore;                      // clip radius (parameter)
  double inv_w;                     // 1 / sigmoid width
  double g;
  double log_floor;
  int n_int;
  int checkpoint;
};

// Queue of molecules that reach the lens entrance with log weight >= floor,
// and (gradient runs) the queue of those still above it after the lens: their
// molecule index and lens-queue slot (which indexes their checkpoints).
struct SoftQueue {
  int32_t* id;
  unsigned int* count;
  unsigned int* max_steps;
  int32_t* bid;
  int32_t* bslot;
  unsigned int* bcount;
  double* bpost;  // gradient runs with planes behind the lens: (5, cap) d lw / d(x, y, vx, vy), d lw / d z0
};

// Per (survivor, segment): the segment's backward map
//   lambda_in = A^T lambda_out + b,  dlw/dV += c . lambda_out + d
// as 25 values A[4][4] (row q = the image of the unit vector e_q), b[4], c[4], d,
// stored as one record of kSoftSegStride values (padded to 16-byte vectors)
// per (survivor, segment), the survivor's segments consecutive: k_soft_compose
// walks a survivor's segments in order and reads each record whole (with the
// 25 values in 25 planes it read 25 scattered sectors per segment).
constexpr int kSoftSegFields = 25;
constexpr int kSoftSegStride = 28;

template <class T>
__device__ __forceinline__ void seg_store(T* o, const T (&v)[kSoftSegStride]) {
  if constexpr (std::is_same<T, float>::value) {
    float4* p = reinterpret_cast<float4*>(o);
#pragma unroll
    for (int k = 0; k < kSoftSegStride / 4; ++k) p[k] = make_float4(v[4 * k], v[4 * k + 1], v[4 * k + 2], v[4 * k + 3]);
  } else {
    double2* p = reinterpret_cast<double2*>(o);
#pragma unroll
    for (int k = 0; k < kSoftSegStride / 2; ++k) p[k] = make_double2(v[2 * k], v[2 * k + 1]);
  }
}

template <class T>
__device__ __forceinline__ void seg_load(const T* o, T (&v)[kSoftSegStride]) {
  if constexpr (std::is_same<T, float>::value) {
    const float4* p = reinterpret_cast<const float4*>(o);
#pragma unroll
    for (int k = 0; k < kSoftSegStride / 4; ++k) {
      const float4 a = __ldg(p + k);
      v[4 * k] = a.x;
      v[4 * k + 1] = a.y;
      v[4 * k + 2] = a.z;
      v[4 * k + 3] = a.w;
    }
  } else {
    const double2* p = reinterpret_cast<const double2*>(o);
#pragma unroll
    for (int k = 0; k < kSoftSegStride / 2; ++k) {
      const double2 a = __ldg(p + k);
      v[2 * k] = a.x;
      v[2 * k + 1] = a.y;
    }
  }
}

// Per-molecule terms (double): weight, then the six gradient terms.  They are
// written to (kSoftAcc, count) columns indexed by molecule and summed in a
// fixed order (k_soft_reduce, then the host), so results do not depend on the
// order in which molecules were queued.
constexpr int kSoftAcc = 1 + kSoftParams;
constexpr int kSoftReduceBlocks = 64;
constexpr int64_t kSoftChunk = int64_t(1) << 22;  // molecules per launch sequence (235 MB of terms)
// soft control block: queue words (256 B), stats, partial column sums
constexpr size_t kSoftCtlBytes = 256 + 8 * kSoftStatCount + 8 * kSoftAcc * kSoftReduceBlocks;

// Column sums in a fixed order: block (b, k) adds rows [b chunk, (b + 1) chunk)
// of column k, thread-strided, then a shared-memory tree.
static __global__ void __launch_bounds__(256) k_soft_reduce(const double* __restrict__ contrib, int64_t count,
                                                     double* __restrict__ partial) {
  __shared__ double s[256];
  const int b = blockIdx.x, k = blockIdx.y;
  const int64_t chunk = (count + gridDim.x - 1) / gridDim.x;
  const int64_t lo = int64_t(b) * chunk, hi = min(count, lo + chunk);
  const double* col = contrib + size_t(k) * size_t(count);
  double v = 0.0;
  for (int64_t r = lo + threadIdx.x; r < hi; r += blockDim.x) v += col[r];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (int(threadIdx.x) < w) s[threadIdx.x] += s[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[size_t(k) * gridDim.x + b] = s[0];
}

template <class T>
struct SoftMol {
  T x, y, vx, vy, vz;
  T nvx, nvy;  // unit normals of vx, vy
  T lw;        // log weight
  T d_ap, d_bore;  // d lw / d aperture radius, d lw / d bore radius

  __device__ void init(const SoftPlan& S, int64_t i) {
    T n0, n1, n2, n3, n4;
    if (S.ic_mode == CTRAJ_IC_DEVICE_DRAW) {
      const Words8 w = molecule_words(S.offset + uint64_t(i), S.key);
      T n5;
      box_muller(w.w[0], w.w[1], n0, n1);
      box_muller(w.w[2], w.w[3], n2, n3);
      box_muller(w.w[4], w.w[5], n4, n5);
    } else {
      const size_t n = size_t(S.n), k = size_t(i);
      n0 = T(S.normals[k]);
      n1 = T(S.normals[n + k]);
      n2 = T(S.normals[2 * n + k]);
      n3 = T(S.normals[3 * n + k]);
      n4 = T(S.normals[4 * n + k]);
    }
    nvx = n0;
    nvy = n1;
    vx = fma_(T(S.s_vx), n0, T(S.mu_vx));
    vy = fma_(T(S.s_vy), n1, T(S.mu_vy));
    vz = fma_(T(S.s_vz), n2, T(S.mu_vz));
    x = mul_(T(S.sx), n3);
    y = mul_(T(S.sy), n4);
    lw = T(0);
    d_ap = T(0);
    d_bore = T(0);
  }

  __device__ T flight_time(const SoftPlan& S, int p) const {
    const double z0 = p == 0 ? S.z_ic : S.z[p - 1];
    return div_(T(S.z[p] - z0), vz);
  }

  // flight to plane p with a = (0, -g)
  __device__ void fly(const SoftPlan& S, int p) {
    const T t = flight_time(S, p);
    const T g = T(S.g);
    x = fma_(vx, t, x);
    y = fma_(mul_(mul_(T(-0.5), g), t), t, fma_(vy, t, y));
    vy = fma_(-g, t, vy);
  }

  // soft edge test at radius R: returns sigma(-z) / w, the derivative of the
  // log weight with respect to R
  __device__ T check(T R, T inv_w) {
    const T r = soft_radius(x, y);
    T ls, dls;
    log_sigmoid(mul_(add_(R, -r), inv_w), ls, dls);
    lw = add_(lw, ls);
    return mul_(dls, inv_w);
  }

  // ballistic part: initial plane to the lens entrance, with the edge tests
  __device__ void front(const SoftPlan& S) {
    const T inv_w = T(S.inv_w);
    for (int p = 0; p < S.n_planes; ++p) {
      fly(S, p);
      if (p == S.n_planes - 1) {
        d_bore = add_(d_bore, check(T(S.bore), inv_w));
      } else if (S.radius[p] < INFINITY) {
        const T d = check(T(S.radius[p]), inv_w);
        if (S.param[p]) d_ap = add_(d_ap, d);
      }
    }
  }
};

template <class T>
__device__ __forceinline__ void accumulate_c(T& s, T& c, T inc) {
  const T d = add_(inc, c);
  const T t = add_(s, d);
  c = add_(d, -add_(t, -s));
  s = t;
}

// One tape entry: the state at the start of a step and the unscaled force
// polynomial P and its slope P' (per table unit) at the four stage points.
template <class T>
struct SoftTape {
  T x, y, vx, vy;
  T P[4], Pp[4];
};

// The lens constants in T, converted once per kernel (a double-to-float
// conversion per use would run on the FP64 pipe inside the step loop).
template <class T>
struct SoftK {
  T beta, neg_s0, kappa, g, kb2, k1;
  int n_int;
  __device__ explicit SoftK(const SoftPlan& S)
      : beta(T(S.beta)), neg_s0(T(-S.s0)), kappa(T(S.kappa)), g(T(S.g)), kb2(T(2.0 * S.kappa * S.beta)),
        k1(T(S.kappa1)), n_int(S.n_int) {}
};

template <class T, bool kStaged>
__device__ __forceinline__ void soft_poly(const SoftK<T>& C, const Coef4<T>* tab, T px, T py, T& P, T& Pp) {
  const T r2 = fma_(py, py, mul_(px, px));
  const T s = fma_(C.beta, r2, C.neg_s0);
  // interval index, clamped (the end pieces extrapolate): truncation to
  // unsigned sends s < 0 and NaN to 0; in FP32 the same index and offset come
  // from table_interval without the conversion unit (a compare-and-select
  // clamp doubled the step's latency; max / min instructions do not)
  unsigned i;
  T u;
  if constexpr (std::is_same<T, float>::value) {
    table_interval(s, unsigned(C.n_int - 1), __int2float_rn(C.n_int - 1), i, u);
  } else {
    i = min(to_uint_rz(s), unsigned(C.n_int - 1));
    u = add_(s, -T(i));
  }
  const Coef4<T> q = tab[i];
  P = fma_(u, fma_(u, q.q2, q.q1), q.q0);
  Pp = fma_(mul_(T(2), u), q.q2, q.q1);
}

// One RK4 step of the lens (the reference's scheme), compensated accumulation;
// with te the state and stage polynomials are written to the tape.
template <class T, bool kStaged>
__device__ __forceinline__ void soft_step(const SoftK<T>& C, const Coef4<T>* tab, T& x, T& y, T& vx, T& vy,
                                          T& cx, T& cy, T& cvx, T& cvy, const T dt, const T hdt, const T c2,
                                          const T dt6, const T dt26, SoftTape<T>* te) {
  const T g = C.g, kappa = C.kappa;
  T P, Pp;
  if (te) { te->x = x; te->y = y; te->vx = vx; te->vy = vy; }
  if constexpr (std::is_same<T, float>::value) {
    // FP32: the (x, y) pairs on the packed FP32 instructions (FFMA2 / FADD2 /
    // FMUL2), per component the same rounding as the scalar path below
    const float2 p = make_float2(x, y), v = make_float2(vx, vy);
    const float2 Hdt = make_float2(hdt, hdt), Dt = make_float2(dt, dt), G0 = make_float2(0.0f, -g);
    auto neg = [](float2 a) { return make_float2(-a.x, -a.y); };
    soft_poly<T, kStaged>(C, tab, x, y, P, Pp);
    if (te) { te->P[0] = P; te->Pp[0] = Pp; }
    float w = mul_(kappa, P);
    const float2 l1 = __ffma2_rn(make_float2(w, w), p, G0);
    const float2 k2 = __ffma2_rn(Hdt, l1, v);
    const float2 p2 = __ffma2_rn(make_float2(c2, c2), v, p);
    soft_poly<T, kStaged>(C, tab, p2.x, p2.y, P, Pp);
    if (te) { te->P[1] = P; te->Pp[1] = Pp; }
    w = mul_(kappa, P);
    const float2 l2 = __ffma2_rn(make_float2(w, w), p2, G0);
    const float2 k3 = __ffma2_rn(Hdt, l2, v);
    const float2 p3 = __ffma2_rn(Hdt, k2, p);
    soft_poly<T, kStaged>(C, tab, p3.x, p3.y, P, Pp);
    if (te) { te->P[2] = P; te->Pp[2] = Pp; }
    w = mul_(kappa, P);
    const float2 l3 = __ffma2_rn(make_float2(w, w), p3, G0);
    const float2 p4 = __ffma2_rn(Dt, k3, p);
    soft_poly<T, kStaged>(C, tab, p4.x, p4.y, P, Pp);
    if (te) { te->P[3] = P; te->Pp[3] = Pp; }
    w = mul_(kappa, P);
    const float2 l4 = __ffma2_rn(make_float2(w, w), p4, G0);
    const float2 sum = __fadd2_rn(__fadd2_rn(l1, l2), l3);
    const float2 dx = __ffma2_rn(make_float2(dt26, dt26), sum, __fmul2_rn(Dt, v));
    const float2 dv = __fmul2_rn(make_float2(dt6, dt6),
                                 __ffma2_rn(make_float2(2.0f, 2.0f), __fadd2_rn(l2, l3), __fadd2_rn(l1, l4)));
    float2 cp = make_float2(cx, cy), cv = make_float2(cvx, cvy);
    const float2 d1 = __fadd2_rn(dx, cp), t1 = __fadd2_rn(p, d1);
    cp = __fadd2_rn(d1, neg(__fadd2_rn(t1, neg(p))));
    const float2 d2 = __fadd2_rn(dv, cv), t2 = __fadd2_rn(v, d2);
    cv = __fadd2_rn(d2, neg(__fadd2_rn(t2, neg(v))));
    x = t1.x;
    y = t1.y;
    vx = t2.x;
    vy = t2.y;
    cx = cp.x;
    cy = cp.y;
    cvx = cv.x;
    cvy = cv.y;
    return;
  }
  soft_poly<T, kStaged>(C, tab, x, y, P, Pp);
  if (te) { te->P[0] = P; te->Pp[0] = Pp; }
  T w = mul_(kappa, P);
  const T l1x = mul_(w, x), l1y = fma_(w, y, -g);
  const T k2x = fma_(hdt, l1x, vx), k2y = fma_(hdt, l1y, vy);
  const T p2x = fma_(c2, vx, x), p2y = fma_(c2, vy, y);
  soft_poly<T, kStaged>(C, tab, p2x, p2y, P, Pp);
  if (te) { te->P[1] = P; te->Pp[1] = Pp; }
  w = mul_(kappa, P);
  const T l2x = mul_(w, p2x), l2y = fma_(w, p2y, -g);
  const T k3x = fma_(hdt, l2x, vx), k3y = fma_(hdt, l2y, vy);
  const T p3x = fma_(hdt, k2x, x), p3y = fma_(hdt, k2y, y);
  soft_poly<T, kStaged>(C, tab, p3x, p3y, P, Pp);
  if (te) { te->P[2] = P; te->Pp[2] = Pp; }
  w = mul_(kappa, P);
  const T l3x = mul_(w, p3x), l3y = fma_(w, p3y, -g);
  const T p4x = fma_(dt, k3x, x), p4y = fma_(dt, k3y, y);
  soft_poly<T, kStaged>(C, tab, p4x, p4y, P, Pp);
  if (te) { te->P[3] = P; te->Pp[3] = Pp; }
  w = mul_(kappa, P);
  const T l4x = mul_(w, p4x), l4y = fma_(w, p4y, -g);
  const T sx = add_(add_(l1x, l2x), l3x);
  const T sy = add_(add_(l1y, l2y), l3y);
  accumulate_c(x, cx, fma_(dt26, sx, mul_(dt, vx)));
  accumulate_c(y, cy, fma_(dt26, sy, mul_(dt, vy)));
  accumulate_c(vx, cvx, mul_(dt6, fma_(T(2), add_(l2x, l3x), add_(l1x, l4x))));
  accumulate_c(vy, cvy, mul_(dt6, fma_(T(2), add_(l2y, l3y), add_(l1y, l4y))));
}

// Transposed Jacobian of one step applied to NV adjoint vectors at once:
// l[v] holds d(.) / d(state after the step) on entry and d(.) / d(state
// before it) on exit; gV[v] gains the step's d(.) / dV.  Stage quantities are
// rebuilt once from the tape entry and shared by the vectors.
template <class T, int NV>
__device__ __forceinline__ void soft_step_adjoint(const SoftK<T>& C, const SoftTape<T>& e, const T dt,
                                                  const T hdt, const T c2, const T dt6, const T dt26,
                                                  T (&l)[NV][4], T (&gV)[NV]) {
  const T g = C.g, kappa = C.kappa, k1 = C.k1, beta = C.beta;
  const T x = e.x, y = e.y, vx = e.vx, vy = e.vy;
  // stage points
  T w = mul_(kappa, e.P[0]);
  const T l1x = mul_(w, x), l1y = fma_(w, y, -g);
  const T k2x = fma_(hdt, l1x, vx), k2y = fma_(hdt, l1y, vy);
  const T p2x = fma_(c2, vx, x), p2y = fma_(c2, vy, y);
  w = mul_(kappa, e.P[1]);
  const T l2x = mul_(w, p2x), l2y = fma_(w, p2y, -g);
  const T k3x = fma_(hdt, l2x, vx), k3y = fma_(hdt, l2y, vy);
  const T p3x = fma_(hdt, k2x, x), p3y = fma_(hdt, k2y, y);
  const T p4x = fma_(dt, k3x, x), p4y = fma_(dt, k3y, y);
  const T px[4] = {x, p2x, p3x, p4x}, py[4] = {y, p2y, p3y, p4y};
  // per stage: w, 2 dw/dr^2 = 2 kappa beta P', dw/dV = kappa1 (P + beta P' r^2)
  T wj[4], dj[4], ej[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    wj[j] = mul_(kappa, e.P[j]);
    dj[j] = mul_(C.kb2, e.Pp[j]);
    const T r2 = fma_(py[j], py[j], mul_(px[j], px[j]));
    ej[j] = mul_(k1, fma_(mul_(beta, e.Pp[j]), r2, e.P[j]));
  }
  // J^T g = w g + (2 dw/dr^2) (p.g) p
  auto stage = [&](int j, T gx, T gy, T& ox, T& oy, T& gv) {
    const T pg = fma_(py[j], gy, mul_(px[j], gx));
    const T f = mul_(dj[j], pg);
    ox = fma_(f, px[j], mul_(wj[j], gx));
    oy = fma_(f, py[j], mul_(wj[j], gy));
    gv = fma_(ej[j], pg, gv);
  };
  const T dt3 = mul_(T(2), dt6), hdt2 = mul_(hdt, hdt), hdtdt = mul_(hdt, dt);
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    const T gx = l[v][0], gy = l[v][1], gvx = l[v][2], gvy = l[v][3];
    T gl1x = fma_(dt26, gx, mul_(dt6, gvx)), gl1y = fma_(dt26, gy, mul_(dt6, gvy));
    T gl2x = fma_(dt26, gx, mul_(dt3, gvx)), gl2y = fma_(dt26, gy, mul_(dt3, gvy));
    const T gl3x = gl2x, gl3y = gl2y;
    const T gl4x = mul_(dt6, gvx), gl4y = mul_(dt6, gvy);
    T lx = gx, ly = gy;
    T lvx = fma_(dt, gx, gvx), lvy = fma_(dt, gy, gvy);
    T ox, oy;
    // stage 4: p4 = x + dt k3, k3 = v + hdt l2
    stage(3, gl4x, gl4y, ox, oy, gV[v]);
    lx = add_(lx, ox);
    ly = add_(ly, oy);
    lvx = fma_(dt, ox, lvx);
    lvy = fma_(dt, oy, lvy);
    gl2x = fma_(hdtdt, ox, gl2x);
    gl2y = fma_(hdtdt, oy, gl2y);
    // stage 3: p3 = x + hdt k2, k2 = v + hdt l1
    stage(2, gl3x, gl3y, ox, oy, gV[v]);
    lx = add_(lx, ox);
    ly = add_(ly, oy);
    lvx = fma_(hdt, ox, lvx);
    lvy = fma_(hdt, oy, lvy);
    gl1x = fma_(hdt2, ox, gl1x);
    gl1y = fma_(hdt2, oy, gl1y);
    // stage 2: p2 = x + c2 v
    stage(1, gl2x, gl2y, ox, oy, gV[v]);
    lx = add_(lx, ox);
    ly = add_(ly, oy);
    lvx = fma_(c2, ox, lvx);
    lvy = fma_(c2, oy, lvy);
    // stage 1: p1 = x
    stage(0, gl1x, gl1y, ox, oy, gV[v]);
    l[v][0] = add_(lx, ox);
    l[v][1] = add_(ly, oy);
    l[v][2] = lvx;
    l[v][3] = lvy;
  }
}

// d lw / d(x, y) of the soft bore test at (x, y): -sigma(-z)/w * (x, y)/r
template <class T>
__device__ __forceinline__ void check_adjoint(T R, T inv_w, T x, T y, T& lx, T& ly) {
  const T r = soft_radius(x, y);
  T ls, dls;
  log_sigmoid(mul_(add_(R, -r), inv_w), ls, dls);
  if (r > T(0)) {
    const T f = div_(mul_(dls, inv_w), r);
    lx = fma_(-f, x, lx);
    ly = fma_(-f, y, ly);
  }
}

// The aperture planes behind the lens: from the state (x, y, vx, vy) after the
// last RK4 step, at zrel = N dz behind the lens entrance, a closed-form flight
// with a = (0, -g) of t_p = (z_p - z0 - zrel) / vz to each plane p, whose soft
// edge test adds to the log weight (and to d_ap for the aperture parameter).
// With lam, d(these log weights) / d(x, y, vx, vy) is added to lam and
// d / d(lens z0) (t_p falls by 1 / vz per unit of z0) to *gz0.
template <class T>
__device__ __forceinline__ void soft_behind(const SoftPlan& S, T x, T y, T vx, T vy, T vz, double zrel, T& lw,
                                            T& d_ap, T* lam, T* gz0) {
  const T inv_w = T(S.inv_w), g = T(S.g);
  for (int p = 0; p < S.n_post; ++p) {
    const double Rd = S.post_radius[p];
    if (!(Rd < INFINITY)) continue;
    const T R = T(Rd);
    const T t = div_(T(S.post_z[p] - S.lens.z0 - zrel), vz);
    const T xp = fma_(vx, t, x);
    const T yp = fma_(mul_(mul_(T(-0.5), g), t), t, fma_(vy, t, y));
    const T r = soft_radius(xp, yp);
    T ls, dls;
    log_sigmoid(mul_(add_(R, -r), inv_w), ls, dls);
    lw = add_(lw, ls);
    if (S.post_param[p]) d_ap = add_(d_ap, mul_(dls, inv_w));
    if (lam && r > T(0)) {
      const T f = div_(mul_(dls, inv_w), r);
      const T gx = mul_(-f, xp), gy = mul_(-f, yp);
      lam[0] = add_(lam[0], gx);
      lam[1] = add_(lam[1], gy);
      lam[2] = fma_(gx, t, lam[2]);
      lam[3] = fma_(gy, t, lam[3]);
      const T vyp = fma_(-g, t, vy);
      *gz0 = add_(*gz0, -div_(fma_(gy, vyp, mul_(gx, vx)), vz));
    }
  }
}

// ---------------------------------------------------------------------------
// k_soft_front: molecules whose weight at the lens entrance is still above
// the floor are queued (by index) with their RK4 step count bound.
template <class T>
__global__ void __launch_bounds__(kThreads) k_soft_front(const __grid_constant__ SoftPlan S, SoftQueue Q,
                                                         unsigned long long* stats) {
  const int lane = threadIdx.x & 31;
  unsigned long long dropped = 0, bad = 0;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  for (int64_t base = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31); base < S.count; base += stride) {
    const int64_t i = S.first + base + lane;
    bool push = false;
    unsigned steps = 0;
    if (base + lane < S.count) {
      SoftMol<T> m;
      m.init(S, i);
      m.front(S);
      if (m.lw >= T(S.log_floor)) {
        LensStep st;
        if (lens_setup(S.lens, double(m.vz), st)) {
          push = true;
          steps = unsigned(st.n_total);
        } else {
          ++bad;
        }
      } else {
        ++dropped;
      }
    }
    const unsigned slot = queue_slot(push, Q.count);
    if (push) Q.id[slot] = int32_t(i);
    const unsigned wmax = __reduce_max_sync(kFull, push ? steps : 0u);
    if (lane == 0 && wmax) atomicMax(Q.max_steps, wmax);
  }
  dropped = warp_sum(dropped);
  bad = warp_sum(bad);
  if (lane == 0) {
    if (dropped) atomicAdd(&stats[kSoftStatDropped], dropped);
    if (bad) atomicAdd(&stats[kSoftStatBad], bad);
  }
}

// ---------------------------------------------------------------------------
// Step parameters of a queued molecule (recomputed from its index).
template <class T>
struct SoftLensSteps {
  int N;
  T dt, hdt, c2, dt6, dt26;
  double zrel;  // N dz: where the last RK4 step ends, from the lens entrance
  __device__ SoftLensSteps(const SoftPlan& S, T vz) {
    LensStep st;
    lens_setup(S.lens, double(vz), st);  // succeeded in k_soft_front
    N = st.n_total;
    zrel = double(N) * st.dz;
    dt = T(st.dt);
    hdt = mul_(T(0.5), dt);
    c2 = S.lens.scheme == CTRAJ_RK4_CLASSIC ? hdt : dt;
    dt6 = mul_(dt, T(1.0 / 6.0));
    dt26 = T(st.dt * st.dt / 6.0);
  }
};

template <class T>
__device__ __forceinline__ void stage_table(const SoftPlan& S, const Coef4<T>* table, Coef4<T>* s_tab) {
  for (int k = threadIdx.x; k < S.n_int; k += blockDim.x) s_tab[k] = table[k];
  __syncthreads();
}

// k_soft_lens: per queued molecule, the lens forward pass: log weight, radius
// derivatives, and with kGrad the checkpoints (state and carried rounding
// errors every K steps; ckpt is (n_seg, 8, cap) values of T, SoA over slots)
// and the queue of molecules that stay above the floor.  The floor test runs
// every 8 steps (the log weight only decreases, so the dropped set is the
// same) to keep it off the step-to-step dependency chain.
template <class T, bool kGrad>
__global__ void __launch_bounds__(kSoftThreads) k_soft_lens(const __grid_constant__ SoftPlan S, const SoftQueue Q,
                                                            const Coef4<T>* __restrict__ table, T* ckpt,
                                                            size_t cap, double* __restrict__ contrib,
                                                            unsigned long long* stats) {
  extern __shared__ unsigned char s_raw[];
  Coef4<T>* s_tab = reinterpret_cast<Coef4<T>*>(s_raw);
  stage_table(S, table, s_tab);
  const unsigned n_in = *Q.count;
  const T inv_w = T(S.inv_w), bore = T(S.bore), floor_ = T(S.log_floor);
  const SoftK<T> C(S);
  const int K = S.checkpoint;
  unsigned long long steps = 0, dropped = 0, entered = 0;
  for (unsigned slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_in; slot += gridDim.x * blockDim.x) {
    const int64_t i = Q.id[slot];
    SoftMol<T> m;
    m.init(S, i);
    m.front(S);
    const SoftLensSteps<T> L(S, m.vz);
    T x = m.x, y = m.y, vx = m.vx, vy = m.vy, cx = T(0), cy = T(0), cvx = T(0), cvy = T(0);
    ++entered;
    bool alive = true;
    int n = 0;
    // One lens step plus the bore test of the state before it (the state
    // after the previous step; the entrance test was done by m.front).  The
    // test does not feed the dynamics.
    auto step = [&](int k) {
      const T qx = x, qy = y;
      soft_step<T, true>(C, s_tab, x, y, vx, vy, cx, cy, cvx, cvy, L.dt, L.hdt, L.c2, L.dt6, L.dt26, nullptr);
      T ls, d;
      soft_test(qx, qy, bore, inv_w, ls, d);
      m.lw = add_(m.lw, k > 0 ? ls : T(0));
      m.d_bore = add_(m.d_bore, k > 0 ? d : T(0));
    };
    auto store_ckpt = [&](int k) {
      T* c = ckpt + size_t(k / K) * 8 * cap + slot;
      c[0] = x; c[cap] = y; c[2 * cap] = vx; c[3 * cap] = vy;
      c[4 * cap] = cx; c[5 * cap] = cy; c[6 * cap] = cvx; c[7 * cap] = cvy;
    };
    if (K % 8 == 0) {
      // Groups of 8 steps without a branch, software-pipelined: a group's
      // steps run beside the bore tests of the previous group's 8 states,
      // which do not depend on them, so the two chains' latencies overlap
      // (with the branch-free FP32 log sigmoid, the slowest molecule's step
      // 550 -> ~370 cycles); the tests are added to the log
      // weight in step order, as one at a time would add them.  The floor
      // test after a group sees the tests up to the previous group: the log
      // weight only decreases, so the same molecules are dropped, up to 8
      // steps later.  Checkpoints between groups.
      T qx[8], qy[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) qx[u] = qy[u] = T(0);
      bool pend = false;  // qx, qy hold the states before steps pn .. pn + 7
      int pn = 0;
      for (; n + 8 <= L.N; n += 8) {
        if (kGrad && n % K == 0) store_ckpt(n);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const T sx = x, sy = y;
          soft_step<T, true>(C, s_tab, x, y, vx, vy, cx, cy, cvx, cvy, L.dt, L.hdt, L.c2, L.dt6, L.dt26, nullptr);
          T ls, d;
          soft_test(qx[u], qy[u], bore, inv_w, ls, d);
          const bool use = pend && pn + u > 0;
          m.lw = add_(m.lw, use ? ls : T(0));
          m.d_bore = add_(m.d_bore, use ? d : T(0));
          qx[u] = sx;
          qy[u] = sy;
        }
        pend = true;
        pn = n;
        if (!(m.lw >= floor_)) {
          alive = false;
          n += 8;
          break;
        }
      }
      if (alive && pend) {  // the last group's tests
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          T ls, d;
          soft_test(qx[u], qy[u], bore, inv_w, ls, d);
          m.lw = add_(m.lw, pn + u > 0 ? ls : T(0));
          m.d_bore = add_(m.d_bore, pn + u > 0 ? d : T(0));
        }
        if (!(m.lw >= floor_)) alive = false;
      }
    }
    for (; alive && n < L.N; ++n) {
      if (kGrad && n % K == 0) store_ckpt(n);
      step(n);
      if ((n & 7) == 7 && !(m.lw >= floor_)) {
        alive = false;
        ++n;
        break;
      }
    }
    if (alive && L.N > 0) {  // the test after the last step
      T ls, d;
      soft_test(x, y, bore, inv_w, ls, d);
      m.lw = add_(m.lw, ls);
      m.d_bore = add_(m.d_bore, d);
    }
    T lam[4] = {T(0), T(0), T(0), T(0)}, gz = T(0);
    if (alive && S.n_post > 0)  // the apertures behind the lens
      soft_behind(S, add_(x, cx), add_(y, cy), add_(vx, cvx), add_(vy, cvy), m.vz, L.zrel, m.lw, m.d_ap,
                  kGrad ? lam : nullptr, &gz);
    if (!(m.lw >= floor_)) alive = false;
    steps += unsigned(n);
    if (!alive) {
      ++dropped;
      continue;
    }
    // this molecule's terms of the sums (row i - first of each column)
    const size_t cnt = size_t(S.count);
    double* o = contrib + size_t(i - S.first);
    const double Tw = exp(double(m.lw));
    o[0] = Tw;
    o[(1 + kSoftAperture) * cnt] = Tw * double(m.d_ap);
    o[(1 + kSoftBore) * cnt] = Tw * double(m.d_bore);
    if (kGrad) {
      const unsigned b = atomicAdd(Q.bcount, 1u);
      Q.bid[b] = int32_t(i);
      Q.bslot[b] = int32_t(slot);
      if (S.n_post > 0) {
#pragma unroll
        for (int q = 0; q < 4; ++q) Q.bpost[size_t(q) * cap + b] = double(lam[q]);
        Q.bpost[4 * cap + b] = double(gz);
      }
    }
  }
  steps = warp_sum(steps);
  dropped = warp_sum(dropped);
  entered = warp_sum(entered);
  if ((threadIdx.x & 31) == 0) {
    if (steps) atomicAdd(&stats[kSoftStatSteps], steps);
    if (dropped) atomicAdd(&stats[kSoftStatDropped], dropped);
    if (entered) atomicAdd(&stats[kSoftStatEntered], entered);
  }
}

// k_soft_seg: one thread per (surviving molecule, lens segment), in parallel
// over segments: recompute the segment from its checkpoint into the tape, then
// run the transposed step Jacobians backwards over it for the four unit
// vectors and the affine part (the segment's own bore tests), giving the
// segment's backward map (A, b, c, d).  seg_out: (bcap * max_seg) records of
// kSoftSegStride values.
template <class T>
__global__ void __launch_bounds__(kSoftThreads) k_soft_seg(const __grid_constant__ SoftPlan S, const SoftQueue Q,
                                                           const Coef4<T>* __restrict__ table,
                                                           const T* __restrict__ ckpt, size_t cap,
                                                           T* __restrict__ seg_out, int max_seg) {
  extern __shared__ unsigned char s_raw[];
  Coef4<T>* s_tab = reinterpret_cast<Coef4<T>*>(s_raw);
  stage_table(S, table, s_tab);
  const size_t n_work = size_t(*Q.bcount) * size_t(max_seg);
  const T inv_w = T(S.inv_w), bore = T(S.bore);
  const SoftK<T> C(S);
  const int K = S.checkpoint;
  for (size_t wi = size_t(blockIdx.x) * blockDim.x + threadIdx.x; wi < n_work; wi += size_t(gridDim.x) * blockDim.x) {
    const size_t b = wi / size_t(max_seg);
    const int sg = int(wi % size_t(max_seg));
    const int32_t slot = Q.bslot[b];
    SoftMol<T> m;
    m.init(S, Q.bid[b]);
    const SoftLensSteps<T> L(S, m.vz);
    const int k0 = sg * K;
    if (k0 >= L.N) continue;
    const int k1 = min(L.N, k0 + K);
    const T* c = ckpt + size_t(sg) * 8 * cap + slot;
    T x = c[0], y = c[cap], vx = c[2 * cap], vy = c[3 * cap];
    T cx = c[4 * cap], cy = c[5 * cap], cvx = c[6 * cap], cvy = c[7 * cap];
    SoftTape<T> tape[kSoftTape];
    for (int k = k0; k < k1; ++k)
      soft_step<T, true>(C, s_tab, x, y, vx, vy, cx, cy, cvx, cvy, L.dt, L.hdt, L.c2, L.dt6, L.dt26,
                         &tape[k - k0]);
    T lam[5][4], gv[5];
#pragma unroll
    for (int v = 0; v < 5; ++v) {
      gv[v] = T(0);
#pragma unroll
      for (int r = 0; r < 4; ++r) lam[v][r] = T(v == r ? 1 : 0);
    }
    // (x, y) is the state after step k1 - 1
    for (int k = k1 - 1; k >= k0; --k) {
      const T ax = k == k1 - 1 ? x : tape[k - k0 + 1].x;
      const T ay = k == k1 - 1 ? y : tape[k - k0 + 1].y;
      check_adjoint(bore, inv_w, ax, ay, lam[4][0], lam[4][1]);
      soft_step_adjoint<T, 5>(C, tape[k - k0], L.dt, L.hdt, L.c2, L.dt6, L.dt26, lam, gv);
    }
    T rec[kSoftSegStride];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
#pragma unroll
      for (int r = 0; r < 4; ++r) rec[q * 4 + r] = lam[q][r];
      rec[20 + q] = gv[q];
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) rec[16 + r] = lam[4][r];
    rec[24] = gv[4];
#pragma unroll
    for (int k = kSoftSegFields; k < kSoftSegStride; ++k) rec[k] = T(0);
    seg_store(seg_out + wi * kSoftSegStride, rec);
  }
}

// k_soft_compose: per surviving molecule, the segments' backward maps applied
// from the last segment to the first, then the ballistic part reversed
// (recomputed): d lw / d(lens z0) from the last flight time, d lw / d(sigma_v)
// from the initial velocities.  Adds the weighted terms to contrib.
template <class T>
__global__ void __launch_bounds__(kSoftThreads) k_soft_compose(const __grid_constant__ SoftPlan S, const SoftQueue Q,
                                                               const T* __restrict__ seg_out, int max_seg,
                                                               double* __restrict__ contrib,
                                                               size_t cap) {
  const unsigned nb = *Q.bcount;
  const T inv_w = T(S.inv_w), bore = T(S.bore);
  for (unsigned b = blockIdx.x * blockDim.x + threadIdx.x; b < nb; b += gridDim.x * blockDim.x) {
    const int64_t i = Q.bid[b];
    SoftMol<T> m;
    m.init(S, i);
    const SoftLensSteps<T> L(S, m.vz);
    const int n_seg = (L.N + S.checkpoint - 1) / S.checkpoint;
    // the adjoint after the lens: the apertures behind it (zero without any)
    T lx = T(0), ly = T(0), lvx = T(0), lvy = T(0), gV = T(0), gz_post = T(0);
    if (S.n_post > 0) {
      lx = T(Q.bpost[b]);
      ly = T(Q.bpost[cap + b]);
      lvx = T(Q.bpost[2 * cap + b]);
      lvy = T(Q.bpost[3 * cap + b]);
      gz_post = T(Q.bpost[4 * cap + b]);
    }
    // unrolled so that the next segments' loads are issued while this one's
    // products wait (a thread walks its segments in order; the maps are read
    // once each)
#pragma unroll 2
    for (int sg = n_seg - 1; sg >= 0; --sg) {
      T o[kSoftSegStride];
      seg_load(seg_out + (size_t(b) * size_t(max_seg) + size_t(sg)) * kSoftSegStride, o);
      const T lo[4] = {lx, ly, lvx, lvy};
      T ln[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) ln[r] = o[16 + r];
      T g = o[24];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
#pragma unroll
        for (int r = 0; r < 4; ++r) ln[r] = fma_(o[q * 4 + r], lo[q], ln[r]);
        g = fma_(o[20 + q], lo[q], g);
      }
      gV = add_(gV, g);
      lx = ln[0];
      ly = ln[1];
      lvx = ln[2];
      lvy = ln[3];
    }
    // the ballistic planes, recomputed, then reversed
    T px[kSoftMaxPlanes], py[kSoftMaxPlanes], pvy[kSoftMaxPlanes];
    for (int p = 0; p < S.n_planes; ++p) {
      m.fly(S, p);
      px[p] = m.x;
      py[p] = m.y;
      pvy[p] = m.vy;
    }
    T gz0 = T(0);
    for (int p = S.n_planes - 1; p >= 0; --p) {
      const T R = p == S.n_planes - 1 ? bore : T(S.radius[p]);
      if (R < T(INFINITY)) check_adjoint(R, inv_w, px[p], py[p], lx, ly);
      const T t = m.flight_time(S, p);
      if (p == S.n_planes - 1) {
        // d t / d z0 = 1 / vz; d x / d t = v at the plane, d vy / d t = -g
        const T gt = fma_(lvy, T(-S.g), fma_(ly, pvy[p], mul_(lx, m.vx)));
        gz0 = add_(div_(gt, m.vz), gz_post);
      }
      lvx = fma_(t, lx, lvx);
      lvy = fma_(t, ly, lvy);
    }
    const size_t cnt = size_t(S.count);
    double* o = contrib + size_t(i - S.first);
    const double Tw = o[0];
    o[(1 + kSoftV) * cnt] = Tw * double(gV);
    o[(1 + kSoftZ0) * cnt] = Tw * double(gz0);
    o[(1 + kSoftSigmaVx) * cnt] = Tw * double(mul_(lvx, m.nvx));
    o[(1 + kSoftSigmaVy) * cnt] = Tw * double(mul_(lvy, m.nvy));
  }
}

}  // namespace ctraj
