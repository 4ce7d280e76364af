// Soft transmission of the lens beamline and its discrete adjoint.
//
// The soft model replaces every hard aperture test of the propagation
// (CircularAperture at its two planes, apertures.py:101-115; the lens
// entrance and the bore test after each RK4 step, electrostatic_lens.py:60-66,
// 112-118) by a sigmoid of the edge distance: a molecule at radius r in front
// of an edge of radius R keeps the weight sigma((R - r) / w), w the sigmoid
// width, and no molecule is removed.  The soft transmission is the mean over
// molecules of the product of all weights, i.e. exp(sum of log-sigmoids); as
// w -> 0 it becomes the detected fraction.  A molecule whose log weight falls
// below `log_floor` (or is not a number) is dropped: its weight, at most
// exp(log_floor), and its gradient are counted as zero.
//
// Parameters (in this order): lens voltage V, lens z0, the radius of one
// circular aperture in front of the lens, the clip radius of the lens bore
// (the field radius stays fixed), and the standard deviations of vx and vy.
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
// -2 alpha / m, alpha = 3 V / R^3.
//
// Gradients are the exact derivatives of this discrete computation (a
// discrete adjoint): the forward pass stores the lens state every
// `checkpoint` steps; the backward pass recomputes each segment from its
// checkpoint into a per-thread tape (state and force polynomial values at the
// four RK4 stage points) and runs the transposed step Jacobians over it in
// reverse, accumulating dlog(T)/dV; the ballistic part is recomputed and
// reversed the same way, giving d/d(lens z0) from the last flight time and
// d/d(sigma_v) from the initial velocities.  The radius derivatives need no
// adjoint (they do not change the dynamics) and are summed in the forward
// pass.
#pragma once
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

template <class T>
struct Coef3 {
  T q0, q1, q2;
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
__device__ __forceinline__ float exp_(float a) { return expf(a); }
__device__ __forceinline__ double exp_(double a) { return exp(a); }
__device__ __forceinline__ float log1p_(float a) { return log1pf(a); }
__device__ __forceinline__ double log1p_(double a) { return log1p(a); }

// log sigma(z) and sigma(-z) = d log sigma(z) / dz
template <class T>
__device__ __forceinline__ void log_sigmoid(T z, T& ls, T& dls) {
  const T e = exp_(z >= T(0) ? -z : z);  // in (0, 1]
  const T l = log1p_(e);
  ls = z >= T(0) ? -l : add_(z, -l);
  dls = z >= T(0) ? div_(e, add_(T(1), e)) : div_(T(1), add_(T(1), e));
}

// Launch-time constants of a soft run.
struct SoftPlan {
  int64_t n;                        // molecules of the whole run
  int64_t first, count;             // the molecules of this launch: first .. first + count - 1
  uint64_t seed, offset;
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
  ctraj_element lens;               // step mode, dz / dt, L (p[7]), scheme
  double V;
  double s0, beta, kappa, kappa1;   // table coordinate and force scales (kappa1 = kappa / V)
  double bore;                      // clip radius (parameter)
  double inv_w;                     // 1 / sigmoid width
  double g;
  double log_floor;
  int n_int;
  int checkpoint;
};

// Queue of molecules that reach the lens entrance with log weight >= floor.
struct SoftQueue {
  int32_t* id;
  unsigned int* count;
  unsigned int* max_steps;
};

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
__global__ void __launch_bounds__(256) k_soft_reduce(const double* __restrict__ contrib, int64_t count,
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
      const Words8 w = molecule_words(S.offset + uint64_t(i), S.seed);
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
    const T r = sqrt_(fma_(y, y, mul_(x, x)));
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

template <class T, bool kStaged>
__device__ __forceinline__ void soft_poly(const SoftPlan& S, const Coef3<T>* tab, T px, T py, T& P, T& Pp) {
  const T r2 = fma_(py, py, mul_(px, px));
  const T s = fma_(T(S.beta), r2, T(-S.s0));
  // interval index, clamped (the end pieces extrapolate); NaN gives the last
  const int i = s >= T(0) ? (s < T(S.n_int) ? int(s) : S.n_int - 1) : (s < T(0) ? 0 : S.n_int - 1);
  const T u = add_(s, -T(i));
  const Coef3<T> q = tab[i];
  P = fma_(u, fma_(u, q.q2, q.q1), q.q0);
  Pp = fma_(mul_(T(2), u), q.q2, q.q1);
}

// One RK4 step of the lens (the reference's scheme), compensated accumulation;
// with te the state and stage polynomials are written to the tape.
template <class T, bool kStaged>
__device__ __forceinline__ void soft_step(const SoftPlan& S, const Coef3<T>* tab, T& x, T& y, T& vx, T& vy,
                                          T& cx, T& cy, T& cvx, T& cvy, const T dt, const T hdt, const T c2,
                                          const T dt6, const T dt26, SoftTape<T>* te) {
  const T g = T(S.g), kappa = T(S.kappa);
  T P, Pp;
  if (te) { te->x = x; te->y = y; te->vx = vx; te->vy = vy; }
  soft_poly<T, kStaged>(S, tab, x, y, P, Pp);
  if (te) { te->P[0] = P; te->Pp[0] = Pp; }
  T w = mul_(kappa, P);
  const T l1x = mul_(w, x), l1y = fma_(w, y, -g);
  const T k2x = fma_(hdt, l1x, vx), k2y = fma_(hdt, l1y, vy);
  const T p2x = fma_(c2, vx, x), p2y = fma_(c2, vy, y);
  soft_poly<T, kStaged>(S, tab, p2x, p2y, P, Pp);
  if (te) { te->P[1] = P; te->Pp[1] = Pp; }
  w = mul_(kappa, P);
  const T l2x = mul_(w, p2x), l2y = fma_(w, p2y, -g);
  const T k3x = fma_(hdt, l2x, vx), k3y = fma_(hdt, l2y, vy);
  const T p3x = fma_(hdt, k2x, x), p3y = fma_(hdt, k2y, y);
  soft_poly<T, kStaged>(S, tab, p3x, p3y, P, Pp);
  if (te) { te->P[2] = P; te->Pp[2] = Pp; }
  w = mul_(kappa, P);
  const T l3x = mul_(w, p3x), l3y = fma_(w, p3y, -g);
  const T p4x = fma_(dt, k3x, x), p4y = fma_(dt, k3y, y);
  soft_poly<T, kStaged>(S, tab, p4x, p4y, P, Pp);
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

// Transposed Jacobian of one step: (lx, ly, lvx, lvy) holds d lw / d(state
// after the step) on entry and d lw / d(state before it) on exit; gV gains the
// step's d lw / dV.  Stage quantities are rebuilt from the tape entry.
template <class T>
__device__ __forceinline__ void soft_step_adjoint(const SoftPlan& S, const SoftTape<T>& e, const T dt,
                                                  const T hdt, const T c2, const T dt6, const T dt26, T& lx,
                                                  T& ly, T& lvx, T& lvy, T& gV) {
  const T g = T(S.g), kappa = T(S.kappa), kb = T(S.kappa * S.beta), k1 = T(S.kappa1), beta = T(S.beta);
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
  // J^T g = w g + 2 (dw/dr^2) (p.g) p;  dw/dr^2 = kappa beta P';  dw/dV = kappa1 (P + beta P' r^2)
  auto stage = [&](int j, T gx, T gy, T& ox, T& oy) {
    const T wj = mul_(kappa, e.P[j]);
    const T dj = mul_(kb, e.Pp[j]);
    const T pg = fma_(py[j], gy, mul_(px[j], gx));
    const T r2 = fma_(py[j], py[j], mul_(px[j], px[j]));
    const T f = mul_(mul_(T(2), dj), pg);
    ox = fma_(f, px[j], mul_(wj, gx));
    oy = fma_(f, py[j], mul_(wj, gy));
    gV = fma_(mul_(k1, fma_(mul_(beta, e.Pp[j]), r2, e.P[j])), pg, gV);
  };
  const T gx = lx, gy = ly, gvx = lvx, gvy = lvy;
  T gl1x = fma_(dt26, gx, mul_(dt6, gvx)), gl1y = fma_(dt26, gy, mul_(dt6, gvy));
  T gl2x = fma_(dt26, gx, mul_(mul_(T(2), dt6), gvx)), gl2y = fma_(dt26, gy, mul_(mul_(T(2), dt6), gvy));
  const T gl3x = gl2x, gl3y = gl2y;
  const T gl4x = mul_(dt6, gvx), gl4y = mul_(dt6, gvy);
  lvx = fma_(dt, gx, gvx);
  lvy = fma_(dt, gy, gvy);
  T ox, oy;
  // stage 4: p4 = x + dt k3, k3 = v + hdt l2
  stage(3, gl4x, gl4y, ox, oy);
  lx = add_(lx, ox);
  ly = add_(ly, oy);
  lvx = fma_(dt, ox, lvx);
  lvy = fma_(dt, oy, lvy);
  gl2x = fma_(mul_(hdt, dt), ox, gl2x);
  gl2y = fma_(mul_(hdt, dt), oy, gl2y);
  // stage 3: p3 = x + hdt k2, k2 = v + hdt l1
  stage(2, gl3x, gl3y, ox, oy);
  lx = add_(lx, ox);
  ly = add_(ly, oy);
  lvx = fma_(hdt, ox, lvx);
  lvy = fma_(hdt, oy, lvy);
  gl1x = fma_(mul_(hdt, hdt), ox, gl1x);
  gl1y = fma_(mul_(hdt, hdt), oy, gl1y);
  // stage 2: p2 = x + c2 v
  stage(1, gl2x, gl2y, ox, oy);
  lx = add_(lx, ox);
  ly = add_(ly, oy);
  lvx = fma_(c2, ox, lvx);
  lvy = fma_(c2, oy, lvy);
  // stage 1: p1 = x
  stage(0, gl1x, gl1y, ox, oy);
  lx = add_(lx, ox);
  ly = add_(ly, oy);
}

// d lw / d(x, y) of the soft bore test at (x, y): -sigma(-z)/w * (x, y)/r
template <class T>
__device__ __forceinline__ void check_adjoint(T R, T inv_w, T x, T y, T& lx, T& ly) {
  const T r = sqrt_(fma_(y, y, mul_(x, x)));
  T ls, dls;
  log_sigmoid(mul_(add_(R, -r), inv_w), ls, dls);
  if (r > T(0)) {
    const T f = div_(mul_(dls, inv_w), r);
    lx = fma_(-f, x, lx);
    ly = fma_(-f, y, ly);
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
// k_soft_lens: per queued molecule, the lens forward pass (log weight, radius
// derivatives, checkpoints when kGrad) and, when kGrad, the backward pass.
// ckpt: (n_seg, 8, cap) values of T, SoA over queue slots.
template <class T, bool kGrad>
__global__ void __launch_bounds__(kSoftThreads) k_soft_lens(const __grid_constant__ SoftPlan S, const SoftQueue Q,
                                                            const Coef3<T>* __restrict__ table, T* ckpt,
                                                            size_t cap, double* __restrict__ contrib,
                                                            unsigned long long* stats) {
  extern __shared__ unsigned char s_raw[];
  Coef3<T>* s_tab = reinterpret_cast<Coef3<T>*>(s_raw);
  for (int k = threadIdx.x; k < S.n_int; k += blockDim.x) s_tab[k] = table[k];
  __syncthreads();
  const unsigned n_in = *Q.count;
  const T inv_w = T(S.inv_w), bore = T(S.bore);
  const bool classic = S.lens.scheme == CTRAJ_RK4_CLASSIC;
  const int K = S.checkpoint;
  unsigned long long steps = 0, dropped = 0, entered = 0;
  for (unsigned slot = blockIdx.x * blockDim.x + threadIdx.x; slot < n_in; slot += gridDim.x * blockDim.x) {
    const int64_t i = Q.id[slot];
    SoftMol<T> m;
    m.init(S, i);
    m.front(S);
    LensStep st;
    lens_setup(S.lens, double(m.vz), st);  // succeeded in k_soft_front
    const int N = st.n_total;
    const T dt = T(st.dt), hdt = mul_(T(0.5), dt);
    const T c2 = classic ? hdt : dt;
    const T dt6 = mul_(dt, T(1.0 / 6.0)), dt26 = T(st.dt * st.dt / 6.0);
    T x = m.x, y = m.y, vx = m.vx, vy = m.vy, cx = T(0), cy = T(0), cvx = T(0), cvy = T(0);
    ++entered;
    bool alive = true;
    int n = 0;
    for (; n < N; ++n) {
      if (kGrad && n % K == 0) {
        T* c = ckpt + size_t(n / K) * 8 * cap + slot;
        c[0] = x; c[cap] = y; c[2 * cap] = vx; c[3 * cap] = vy;
        c[4 * cap] = cx; c[5 * cap] = cy; c[6 * cap] = cvx; c[7 * cap] = cvy;
      }
      soft_step<T, true>(S, s_tab, x, y, vx, vy, cx, cy, cvx, cvy, dt, hdt, c2, dt6, dt26, nullptr);
      m.x = x;
      m.y = y;
      m.d_bore = add_(m.d_bore, m.check(bore, inv_w));
      if (!(m.lw >= T(S.log_floor))) {
        alive = false;
        ++n;
        break;
      }
    }
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
    if (!kGrad) continue;
    // ---- backward through the lens, segment by segment
    T lx = T(0), ly = T(0), lvx = T(0), lvy = T(0), gV = T(0);
    SoftTape<T> tape[kSoftTape];
    const int n_seg = (N + K - 1) / K;
    for (int sg = n_seg - 1; sg >= 0; --sg) {
      const T* c = ckpt + size_t(sg) * 8 * cap + slot;
      x = c[0]; y = c[cap]; vx = c[2 * cap]; vy = c[3 * cap];
      cx = c[4 * cap]; cy = c[5 * cap]; cvx = c[6 * cap]; cvy = c[7 * cap];
      const int k0 = sg * K, k1 = min(N, k0 + K);
      for (int k = k0; k < k1; ++k)
        soft_step<T, true>(S, s_tab, x, y, vx, vy, cx, cy, cvx, cvy, dt, hdt, c2, dt6, dt26, &tape[k - k0]);
      // (x, y) is the state after step k1 - 1
      for (int k = k1 - 1; k >= k0; --k) {
        const T ax = k == k1 - 1 ? x : tape[k - k0 + 1].x;
        const T ay = k == k1 - 1 ? y : tape[k - k0 + 1].y;
        check_adjoint(bore, inv_w, ax, ay, lx, ly);
        soft_step_adjoint(S, tape[k - k0], dt, hdt, c2, dt6, dt26, lx, ly, lvx, lvy, gV);
      }
    }
    // ---- backward through the ballistic planes (recomputed)
    SoftMol<T> b;
    b.init(S, i);
    T px[kSoftMaxPlanes], py[kSoftMaxPlanes], pvy[kSoftMaxPlanes];
    for (int p = 0; p < S.n_planes; ++p) {
      b.fly(S, p);
      px[p] = b.x;
      py[p] = b.y;
      pvy[p] = b.vy;
    }
    T gz0 = T(0);
    for (int p = S.n_planes - 1; p >= 0; --p) {
      const T R = p == S.n_planes - 1 ? bore : T(S.radius[p]);
      if (R < T(INFINITY)) check_adjoint(R, inv_w, px[p], py[p], lx, ly);
      const T t = b.flight_time(S, p);
      if (p == S.n_planes - 1) {
        // d t / d z0 = 1 / vz; d x / d t = v at the plane, d vy / d t = -g
        const T gt = fma_(lvy, T(-S.g), fma_(ly, pvy[p], mul_(lx, b.vx)));
        gz0 = div_(gt, b.vz);
      }
      lvx = fma_(t, lx, lvx);
      lvy = fma_(t, ly, lvy);
    }
    o[(1 + kSoftV) * cnt] = Tw * double(gV);
    o[(1 + kSoftZ0) * cnt] = Tw * double(gz0);
    o[(1 + kSoftSigmaVx) * cnt] = Tw * double(mul_(lvx, m.nvx));
    o[(1 + kSoftSigmaVy) * cnt] = Tw * double(mul_(lvy, m.nvy));
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

}  // namespace ctraj
