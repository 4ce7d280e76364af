// Per-molecule state and element physics, in two precisions.
//
// Mol64 follows the reference's float64 operation order step for step, using
// __dadd_rn/__dmul_rn (never contracted into FMA) and IEEE division and square
// root, so on ballistic paths it reproduces the reference bit for bit:
//   update_trajectory    molecule.py:26-68
//   aperture hit tests   apertures.py:101-115, 174-189
//   field plates         apertures.py:227-270
//   lens force           electrostatic_lens.py:215-227 with scipy's PPoly
//                        (nu = 1) or numpy.interp evaluation order
//   lens RK4 step        electrostatic_lens.py:91-118
//
// Mol32 restates the same physics for speed.  The molecule always sits on the
// last plane it reached, so a flight is (plane gap) * (1/vz) with the gap
// precomputed in double on the host; z itself is never accumulated in float.
// Inside the lens only the transverse state (x, y, vx, vy) evolves (a_z = 0)
// and the force is a_perp = w(|r|) * (x, y) - g y^, w read from a per-interval
// polynomial table.  The RK4 combination is rewritten exactly:
//   x' = x + dt v + dt^2/6 (l1 + l2 + l3),  v' = v + dt/6 (l1 + 2 l2 + 2 l3 + l4)
// (the reference's k1..k4 substituted); each increment is formed in full
// precision and added with a carried rounding error (compensated summation),
// and the step count, step size and exit-snap time are computed once per
// molecule in double.
#pragma once
#include <cfloat>
#include <cmath>
#include <cstdint>

#include "philox.cuh"
#include "plan.cuh"

namespace ctraj {

__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// ---------------------------------------------------------------------------
// FP64 force table lookups (reference evaluation order)
// ---------------------------------------------------------------------------

// scipy PPoly.__call__(E, nu=1): interval knots[i] <= E < knots[i+1], end
// pieces extrapolated; res = 0 + c2*1*1; res += (c1*s)*2; res += (c0*(s*s))*3.
__device__ inline double spline_deriv64(const TableD& T, double E, int& range) {
  const int n = T.n;
  int i;
  if (isnan(E)) return E;
  if (E < T.x0) {
    i = 0;
    range = 1;
  } else if (E >= __ldg(T.knots + n - 1)) {
    i = n - 2;
    if (E > __ldg(T.knots + n - 1)) range = 1;
  } else {
    i = int(floor((E - T.x0) / T.h));
    i = max(0, min(i, n - 2));
    while (i > 0 && E < __ldg(T.knots + i)) --i;
    while (i < n - 2 && E >= __ldg(T.knots + i + 1)) ++i;
  }
  const double* c = T.coef + 4 * size_t(i);
  const double s = dadd(E, -__ldg(T.knots + i));
  double res = 0.0;
  res = dadd(res, dmul(dmul(__ldg(c + 2), 1.0), 1.0));
  res = dadd(res, dmul(dmul(__ldg(c + 1), s), 2.0));
  res = dadd(res, dmul(dmul(__ldg(c + 0), dmul(s, s)), 3.0));
  return res;
}

// numpy.interp(r, knots, values) (what scipy's float64 linear interp1d calls),
// with interp1d's bounds error above the last knot reported through err.
__device__ inline double radial64(const TableD& T, double r, int& err) {
  const int n = T.n;
  const double last = __ldg(T.knots + n - 1);
  if (r < T.x0 || r > last) {
    err = 1;
    return nan("");
  }
  if (isnan(r)) return r;
  int j = int(floor((r - T.x0) / T.h));
  j = max(0, min(j, n - 1));
  while (j > 0 && __ldg(T.knots + j) > r) --j;
  while (j < n - 1 && __ldg(T.knots + j + 1) <= r) ++j;
  const double xj = __ldg(T.knots + j), yj = __ldg(T.values + j);
  if (j == n - 1 || xj == r) return yj;
  const double slope = (__ldg(T.values + j + 1) - yj) / (__ldg(T.knots + j + 1) - xj);
  return dadd(dmul(slope, dadd(r, -xj)), yj);
}

// ElectrostaticLens.lens_acceleration (electrostatic_lens.py:215-227).
__device__ inline void lens_force64(const Plan& P, const ctraj_element& e, double x0, double x1,
                                    double& a0, double& a1, int& range, int& err) {
  const TableD& T = P.td[e.table];
  const double r = __dsqrt_rn(dadd(dmul(x0, x0), dmul(x1, x1)));
  double a_r;
  if (T.kind == CTRAJ_TABLE_RADIAL_LINEAR) {
    a_r = radial64(T, r, err);
  } else {
    const double alpha = e.p[6], mass = e.p[5];
    if (e.field_order == 1) {
      const double E = dmul(alpha, r);
      a_r = -dmul(spline_deriv64(T, E, range), alpha) / mass;
    } else {
      const double E = dmul(alpha, dmul(r, r));
      a_r = -dmul(spline_deriv64(T, E, range), dmul(dmul(2.0, alpha), r)) / mass;
    }
  }
  a0 = 0.0;
  a1 = 0.0;
  if (r != 0.0) {
    a0 = dmul(a_r, x0) / r;
    a1 = dmul(a_r, x1) / r;
  }
  a1 = dadd(a1, -P.g);
}

// ---------------------------------------------------------------------------
// Honeycomb nearest cell (meshes.py:104-108)
// ---------------------------------------------------------------------------
// The reference takes numpy's argmin over ALL centres of
// sqrt((px - xc)**2 + (py - yc)**2): the first of equal minima, 0 when no
// distance is finite.  The centres form hexalattice rows of nx cells (odd rows
// shifted by half a pitch), so the nearest centre of an interior point is at
// most one row and one cell from the rounded estimate, and the second-nearest
// at most two.  Outside the grid the estimate is clamped; the nearest and
// second-nearest centres of a point beyond the first or last row are among
// the outermost four rows (the nearest of each row is its cell closest in x,
// and rows alternate their half-pitch shift), so the window takes rows
// j0-2..j0+2, widened to four rows at either end, and cells i0-2..i0+2 of each.
// Scanning the window rows and cells in ascending order visits cells in
// ascending index, so strict < keeps the first minimum as argmin does.

// rows of the search window around the (clamped) estimate j0 of ny rows
__device__ __forceinline__ void window_rows(int j0, int ny, int& lo, int& hi) {
  lo = j0 == ny - 1 ? max(ny - 4, 0) : max(j0 - 2, 0);
  hi = j0 == 0 ? min(3, ny - 1) : min(j0 + 2, ny - 1);
}

// round(u) clamped to [0, hi]; NaN -> 0
__device__ __forceinline__ int window_index(double u, int hi) {
  const double r = floor(u + 0.5);
  if (!(r >= 0.0)) return 0;
  return r >= double(hi) ? hi : int(r);
}

// FP64, the reference's operations; best / second: the two smallest distances.
__device__ inline int mesh_nearest64(const TableD& T, const double* p, double px, double py, double& best,
                                     double& second) {
  const int nx = int(p[1]), ny = T.n / nx;
  const int j0 = window_index((py - __ldg(T.values)) * p[2], ny - 1);
  int lo, hi;
  window_rows(j0, ny, lo, hi);
  int idx = -1;
  best = INFINITY;
  second = INFINITY;
  for (int j = lo; j <= hi; ++j) {
    const int row = j * nx;
    const int i0 = window_index((px - __ldg(T.knots + row)) * p[3], nx - 1);
    for (int k = row + max(i0 - 2, 0); k <= row + min(i0 + 2, nx - 1); ++k) {
      const double dx = dadd(px, -__ldg(T.knots + k)), dy = dadd(py, -__ldg(T.values + k));
      const double d = __dsqrt_rn(dadd(dmul(dx, dx), dmul(dy, dy)));
      if (d < best) {
        second = best;
        best = d;
        idx = k;
      } else if (d < second) {
        second = d;
      }
    }
  }
  return idx < 0 ? 0 : idx;
}

// FP32 on the float4 (x, y, 0, 0) centre table; squared distances.
__device__ __forceinline__ int window_index32(float u, int hi) {
  const float r = floorf(u + 0.5f);
  if (!(r >= 0.0f)) return 0;
  return r >= float(hi) ? hi : int(r);
}

__device__ inline int mesh_nearest32(const LensF& L, const ElemF& f, float px, float py, float& best2,
                                     float& second2) {
  const int nx = L.cols, ny = L.n_int / nx;
  const int j0 = window_index32((py - __ldg(&L.q[0].y)) * f.c[2], ny - 1);
  int lo, hi;
  window_rows(j0, ny, lo, hi);
  int idx = -1;
  best2 = INFINITY;
  second2 = INFINITY;
  for (int j = lo; j <= hi; ++j) {
    const int row = j * nx;
    const int i0 = window_index32((px - __ldg(&L.q[row].x)) * f.c[3], nx - 1);
    for (int k = row + max(i0 - 2, 0); k <= row + min(i0 + 2, nx - 1); ++k) {
      const float4 c = __ldg(L.q + k);
      const float dx = px - c.x, dy = py - c.y;
      const float d2 = __fmaf_rn(dy, dy, __fmul_rn(dx, dx));
      if (d2 < best2) {
        second2 = best2;
        best2 = d2;
        idx = k;
      } else if (d2 < second2) {
        second2 = d2;
      }
    }
  }
  return idx < 0 ? 0 : idx;
}

// ---------------------------------------------------------------------------
// FP32 table interval: i = min(trunc_to_unsigned(s), last) and u = s - i, as
// the truncating float-to-unsigned conversion and its inverse give them
// (negative and NaN s -> interval 0; u keeps s's own offset), without the
// conversion unit: 2^23 + max(s, 0) rounded toward -inf is 2^23 + floor(s)
// for s < 2^23 (the spacing of floats in [2^23, 2^24) is 1), so floor(s)
// sits in the low mantissa bits and 2^23 subtracts back exactly; larger s
// and infinity land on the clamp.  Bit-identical to the conversions, on
// FP32 / integer pipes instead of the conversion pipe.  The soft-transmission
// kernels (4 % faster) and the linear-table lens lookups (one warp's step
// 323 -> 231 cycles) use it; the quadratic-table lookups keep the
// conversions, which measured as fast there.
// kNonNeg: s is known to be >= 0 or NaN (a linear Stark table starts at
// |E| = 0 and its coordinate scale is not negative), so max(s, 0) is left
// out; only a NaN s then takes the last interval instead of the first, and
// u, hence the force, is NaN either way.
// ---------------------------------------------------------------------------
template <bool kNonNeg = false>
__device__ __forceinline__ void table_interval(const float s, const unsigned last, const float last_f,
                                               unsigned& i, float& u) {
  const float t = __fadd_rd(kNonNeg ? s : fmaxf(s, 0.0f), 8388608.0f);
  i = min(__float_as_uint(t) - 0x4B000000u, last);
  u = __fadd_rn(s, -fminf(__fadd_rn(t, -8388608.0f), last_f));
}

// ---------------------------------------------------------------------------
// FP32 force: w such that a_perp = w * (x, y)
// ---------------------------------------------------------------------------
// kStaged: the whole table is in shared memory (s_tab); otherwise it is read
// from global memory through the read-only cache.  Lookups past the last
// interval extrapolate it (as scipy CubicSpline does); s < 0 uses interval 0.
// `beta` is the table-coordinate scale (L.beta, or a molecule's own in a
// batched sweep where each configuration has its lens voltage).
// kScaled: beta is a molecule's own (a batched sweep's configuration), not
// the table's L.beta, which the host checked to be >= 0.
template <int F, bool kStaged, bool kScaled = false>
__device__ __forceinline__ float wforce(float px, float py, const LensArgs& L, const float4* s_tab,
                                        unsigned& flags, const float beta) {
  const float r2 = __fmaf_rn(py, py, __fmul_rn(px, px));
  if (F == kForceStark2Lin) {
    // quarter-interval piece (w, dw): one 8-byte lookup, ~5.4 bank-conflicted
    // shared-memory wavefronts per warp instead of ~9 for the 16-byte
    // quadratic entry; s counts pieces, the table holds 2 * n_int of them
    const float s = __fmaf_rn(beta, r2, -L.s0);
    // (the interval without the conversion unit: one warp's RK4 step 231
    // instead of 323 cycles, bit-identical)
    unsigned i;
    float u;
    // s >= 0: the linear form's table starts at |E| = 0 (s0 <= 0) and L.beta >= 0
    table_interval<!kScaled>(s, unsigned(2 * L.n_int - 1), __int2float_rn(2 * L.n_int - 1), i, u);
    const float2 q = kStaged ? reinterpret_cast<const float2*>(s_tab)[i]
                             : __ldg(reinterpret_cast<const float2*>(L.q) + i);
    return __fmaf_rn(u, q.y, q.x);
  }
  float s, r = 0.0f;
  if (F == kForceStark2) {
    s = __fmaf_rn(beta, r2, -L.s0);
  } else {
    r = sqrtf(r2);
    s = __fmaf_rn(beta, r, -L.s0);
    if (F == kForceRadial) flags |= (r > L.r_max) ? 2u : 0u;
  }
  const unsigned i = min(__float2uint_rz(s), unsigned(L.n_int - 1));  // negative s -> 0
  const float u = __fadd_rn(s, -__uint2float_rn(i));
  const float4 q = kStaged ? s_tab[i] : __ldg(L.q + i);
  if (F == kForceRadial) {
    const float a_r = __fmaf_rn(u, q.y, q.x);
    return r > 0.0f ? __fdividef(a_r, r) : 0.0f;
  }
  const float w = __fmaf_rn(u, __fmaf_rn(u, q.z, q.y), q.x);
  if (F == kForceStark1) return r > 0.0f ? __fdividef(w, r) : 0.0f;
  return w;
}

// Per-molecule lens integration parameters (both precisions).
struct LensStep {
  int n_total;  // rint(L/dz), at most CTRAJ_MAX_LENS_STEPS; -1 while the setup is pending
  int n_done;
  int bound;    // upper bound on n_total while the setup is pending
  double dt;        // dz / vz
  double snap;      // FP32: exit-snap time (z1 - z0 - N dz) / vz
  double dz;
};

// Step count and step size exactly as electrostatic_lens.py:87-88, in double.
__device__ __forceinline__ bool lens_setup(const ctraj_element& e, double vz, LensStep& s) {
  const double dz = e.step_mode == CTRAJ_STEP_DT ? dmul(vz, e.p[2]) : e.p[1];
  const double nf = rint(e.p[7] / dz);
  s.dz = dz;
  s.n_done = 0;
  if (!(fabs(nf) <= double(CTRAJ_MAX_LENS_STEPS))) {  // also catches NaN / inf
    s.n_total = 0;
    s.dt = 0.0;
    s.snap = 0.0;
    return false;
  }
  s.n_total = nf < 0.0 ? 0 : int(nf);
  s.dt = dz / vz;
  s.snap = ((e.z1 - e.z0) - double(s.n_total) * dz) / vz;
  return true;
}

// Trajectory row sink used by the replay kernel.
struct RowSink {
  double* out;   // (max_rows, 10)
  int max_rows;
  int stride;
  int64_t row;   // index of the last stored row (0 = initial)
  int written;
  bool last_written;
  // Plane mode (stride 1, out unused): follow the rows to the crossing of the
  // plane z = zp the way post_processing.py:37-76 reads a trajectory: the first
  // row anywhere with z == zp (pexact; the lens's last steps can overshoot z1
  // and the exit snap come back to it), else the row before the first one with
  // z >= zp (pcross = 2; 3 when that is the first row: Python's index -1, the
  // last row); rows with a non-finite value are skipped, as drop_nans
  // (molecule.py:160-167) removes them.
  bool plane;
  bool pexact;
  int pcross;
  double zp;
  double prev[10], hit[10], last[10], exact[10];
  __device__ void put(double x, double y, double z, double vx, double vy, double vz, double ax,
                      double ay, double az, double t) {
    ++row;
    last_written = false;
    if (row % stride == 0) write(x, y, z, vx, vy, vz, ax, ay, az, t);
  }
  __device__ void write(double x, double y, double z, double vx, double vy, double vz, double ax,
                        double ay, double az, double t) {
    if (plane) {
      const double r[10] = {x, y, z, vx, vy, vz, ax, ay, az, t};
      bool finite = true;
      for (int k = 0; k < 10; ++k) finite = finite && isfinite(r[k]);
      if (finite) {
        if (!pexact && z == zp) {
          for (int k = 0; k < 10; ++k) exact[k] = r[k];
          pexact = true;
        }
        if (pcross == 0 && !(z < zp)) {
          if (written == 0) {
            pcross = 3;
          } else {
            for (int k = 0; k < 10; ++k) hit[k] = prev[k];
            pcross = 2;
          }
        }
        for (int k = 0; k < 10; ++k) prev[k] = last[k] = r[k];
        ++written;
      }
      last_written = true;
      return;
    }
    if (written < max_rows) {
      double* o = out + size_t(written) * 10;
      o[0] = x; o[1] = y; o[2] = z; o[3] = vx; o[4] = vy; o[5] = vz;
      o[6] = ax; o[7] = ay; o[8] = az; o[9] = t;
    }
    ++written;
    last_written = true;
  }
};

// ===========================================================================
// FP64: the reference's arithmetic
// ===========================================================================
template <bool kRec>
struct Mol64 {
  static constexpr bool kScreenable = false;  // the front's screening is FP32's (Mol32)
  double x[3], v[3], a[3], t;
  double margin;
  int rows;
  int32_t id;
  RowSink* sink;

  __device__ void row_out() {
    if (kRec) sink->put(x[0], x[1], x[2], v[0], v[1], v[2], a[0], a[1], a[2], t);
  }

  __device__ void init(const Plan& P, const RunDev& R, int64_t i) {
    id = int32_t(i);
    margin = INFINITY;
    rows = 0;
    if (R.ic_mode == CTRAJ_IC_DEVICE_DRAW) {
      const Words8 w = molecule_words(R.offset + uint64_t(i), R.key);
      double n0, n1, n2, n3, n4, n5;
      box_muller(w.w[0], w.w[1], n0, n1);
      box_muller(w.w[2], w.w[3], n2, n3);
      box_muller(w.w[4], w.w[5], n4, n5);
      const double* vp = R.vd.p;
      v[0] = __fma_rn(vp[1], n0, vp[0]);
      v[1] = __fma_rn(vp[3], n1, vp[2]);
      v[2] = __fma_rn(vp[5], n2, vp[4]);
      const double* xp = R.xd.p;
      if (R.xd.kind == CTRAJ_DIST_DISC_POSITION) {
        double s, c;
        sincospi(2.0 * u01d(w.w[6]), &s, &c);
        const double rr = dmul(sqrt(u01d(w.w[7])), dmul(xp[0], 0.5));
        x[0] = dmul(rr, c);
        x[1] = dmul(rr, s);
        x[2] = xp[1];
      } else {
        x[0] = dmul(xp[0], n3);
        x[1] = dmul(xp[1], n4);
        x[2] = xp[2];
      }
    } else {
      const size_t n = size_t(R.n);
      for (int k = 0; k < 3; ++k) {
        x[k] = R.ics[k * n + size_t(i)];
        v[k] = R.ics[(3 + k) * n + size_t(i)];
      }
    }
    a[0] = 0.0;
    a[1] = -P.g;
    a[2] = 0.0;
    t = 0.0;
    if (kRec) sink->write(x[0], x[1], x[2], v[0], v[1], v[2], a[0], a[1], a[2], t);
  }

  // Molecule.update_trajectory(delta_t, a=(0,-g,0))
  __device__ void update(double dt, const Plan& P) {
    if (dt != 0.0) {  // `if not delta_t` keeps x and v (molecule.py:31,41)
      const double dt2 = dmul(dt, dt);
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        x[k] = dadd(dadd(x[k], dmul(v[k], dt)), dmul(dmul(a[k], dt2), 0.5));
        v[k] = dadd(v[k], dmul(a[k], dt));
      }
    }
    t = dadd(t, dt);
    a[0] = 0.0;
    a[1] = -P.g;
    a[2] = 0.0;
    rows += isfinite(t) ? 1 : 0;
    row_out();
  }

  __device__ void fly(const Plan& P, int i, int which) {
    const double z = which ? P.el[i].z1 : P.el[i].z0;
    update((z - x[2]) / v[2], P);
  }

  __device__ double rho() const { return __dsqrt_rn(dadd(dmul(x[0], x[0]), dmul(x[1], x[1]))); }

  __device__ void note(double d) { margin = fmin(margin, fabs(d)); }

  __device__ bool circle_out(const Plan& P, int i) {
    const double r = rho(), h = dmul(P.el[i].p[0], 0.5);
    note(dadd(r, -h));
    return r > h;
  }
  __device__ bool rect_out(const Plan& P, int i) {
    const double* p = P.el[i].p;
    note(dadd(x[0], -p[0])); note(dadd(x[0], -p[1])); note(dadd(x[1], -p[2])); note(dadd(x[1], -p[3]));
    return !((p[0] < x[0] && x[0] < p[1]) && (p[2] < x[1] && x[1] < p[3]));
  }
  // FieldPlates after the z0 flight: returns true when lost (apertures.py:238-270)
  __device__ bool plates(const Plan& P, int i) {
    const double x1 = P.el[i].p[0], x2 = P.el[i].p[1];
    note(dadd(x[0], -x1)); note(dadd(x[0], -x2));
    if (!(x1 < x[0] && x[0] < x2)) return true;
    double dt = (P.el[i].z1 - x[2]) / v[2];
    const double xe = dt != 0.0 ? dadd(dadd(x[0], dmul(v[0], dt)), dmul(dmul(a[0], dmul(dt, dt)), 0.5)) : x[0];
    note(dadd(xe, -x1)); note(dadd(xe, -x2));
    if (!(x1 < xe && xe < x2)) {
      if (v[0] < 0) dt = (x1 - x[0]) / v[0];
      else if (v[0] > 0) dt = (x2 - x[0]) / v[0];
      update(dt, P);
      return true;
    }
    update(dt, P);
    return false;
  }
  // Honeycomb test at the plane just reached (meshes.py:98-116): cell = the
  // nearest centre, looked up while it is None or 0 (`if not idx`); lost when
  // outside that cell's hexagon, |dx| < R sqrt(3)/2 and |dy| < R - |dx|/sqrt(3).
  // Margins: half the gap between nearest and second-nearest centre, and the
  // nearer hexagon side.
  __device__ bool honeycomb_out(const Plan& P, int i, int& cell) {
    const ctraj_element& e = P.el[i];
    const TableD& T = P.td[e.table];
    if (cell <= 0) {
      double best, second;
      cell = mesh_nearest64(T, e.p, x[0], x[1], best, second);
      note(dadd(second, -best) / 2.0);
    }
    const double s3 = __dsqrt_rn(3.0), R = e.p[0];
    const double dx = fabs(dadd(x[0], -__ldg(T.knots + cell))), dy = fabs(dadd(x[1], -__ldg(T.values + cell)));
    const double hw = dmul(R, s3) / 2.0, q = __ddiv_rn(dx, s3);
    const double side = dadd(hw, -dx), slant = dmul(dadd(dadd(R, -q), -dy), s3 / 2.0);
    note(side < slant ? side : slant);
    return !(dx < hw && dy < dadd(R, -q));
  }

  __device__ bool lens_entrance_out(const Plan& P, int i) { return circle_out(P, i); }

  __device__ double vel_z() const { return v[2]; }

  // One reference RK4 step (electrostatic_lens.py:91-118); returns true when lost.
  __device__ bool lens_step(const Plan& P, int i, const LensStep& s, int& range, int& err) {
    const ctraj_element& e = P.el[i];
    const double dt = s.dt;
    const bool classic = e.scheme == CTRAJ_RK4_CLASSIC;
    double k1[3], l1[3], k2[3], l2[3], k3[3], l3[3], k4[3], l4[3], p[3];
    for (int k = 0; k < 3; ++k) k1[k] = v[k];
    lens_force64(P, e, x[0], x[1], l1[0], l1[1], range, err);
    l1[2] = 0.0;
    for (int k = 0; k < 3; ++k) {
      k2[k] = dadd(k1[k], dmul(dmul(dt, l1[k]), 0.5));
      p[k] = classic ? dadd(x[k], dmul(dmul(dt, k1[k]), 0.5)) : dadd(x[k], dmul(dt, k1[k]));
    }
    lens_force64(P, e, p[0], p[1], l2[0], l2[1], range, err);
    l2[2] = 0.0;
    for (int k = 0; k < 3; ++k) {
      k3[k] = dadd(k1[k], dmul(dmul(dt, l2[k]), 0.5));
      p[k] = dadd(x[k], dmul(dmul(dt, k2[k]), 0.5));
    }
    lens_force64(P, e, p[0], p[1], l3[0], l3[1], range, err);
    l3[2] = 0.0;
    for (int k = 0; k < 3; ++k) {
      k4[k] = dadd(k1[k], dmul(dt, l3[k]));
      p[k] = dadd(x[k], dmul(dt, k3[k]));
    }
    lens_force64(P, e, p[0], p[1], l4[0], l4[1], range, err);
    l4[2] = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double sk = dadd(dadd(dadd(k1[k], dmul(2.0, k2[k])), dmul(2.0, k3[k])), k4[k]);
      const double sl = dadd(dadd(dadd(l1[k], dmul(2.0, l2[k])), dmul(2.0, l3[k])), l4[k]);
      x[k] = dadd(x[k], dmul(dt, sk) / 6.0);
      v[k] = dadd(k1[k], dmul(dt, sl) / 6.0);
      a[k] = l1[k];
    }
    t = dadd(t, dt);
    rows += isfinite(t) ? 1 : 0;
    row_out();
    if (err) return true;
    const double r = rho(), h = dmul(e.p[0], 0.5);
    note(dadd(r, -h));
    return r > h;
  }

  __device__ void lens_begin(const Plan&, int, const LensStep&) {}
  __device__ void lens_row(const Plan&, int, const LensStep&) {}
  // After the last step: the exit snap with the stored acceleration l1
  // (electrostatic_lens.py:74-77) unless the molecule was lost inside.
  __device__ void lens_end(const Plan& P, int i, const LensStep&, bool lost) {
    if (!lost) fly(P, i, 1);
  }

  __device__ void final_row(double* f, int64_t i, int64_t n) const {
    const double vals[10] = {x[0], x[1], x[2], v[0], v[1], v[2], a[0], a[1], a[2], t};
    for (int k = 0; k < 10; ++k) f[size_t(k) * size_t(n) + size_t(i)] = vals[k];
  }
  __device__ void flush_last() {
    if (kRec && !sink->last_written) sink->write(x[0], x[1], x[2], v[0], v[1], v[2], a[0], a[1], a[2], t);
  }

  __device__ void store(const Queue& Q, unsigned s, const LensStep& st) const {
    Q.dx[s] = x[0]; Q.dy[s] = x[1]; Q.dz[s] = x[2];
    Q.dvx[s] = v[0]; Q.dvy[s] = v[1]; Q.dvz[s] = v[2];
    Q.dt[s] = t; Q.margin[s] = margin; Q.rows[s] = rows; Q.id[s] = id;
    Q.lens_dt[s] = st.dt; Q.n_done[s] = int32_t(st.n_done); Q.n_total[s] = int32_t(st.n_total);
  }
  // The stored acceleration is not carried: the next RK4 step recomputes it.
  __device__ void load_state(const Queue& Q, unsigned s, const Plan& P, LensStep& st) {
    x[0] = Q.dx[s]; x[1] = Q.dy[s]; x[2] = Q.dz[s];
    v[0] = Q.dvx[s]; v[1] = Q.dvy[s]; v[2] = Q.dvz[s];
    t = Q.dt[s]; margin = Q.margin[s]; rows = Q.rows[s]; id = Q.id[s];
    a[0] = 0.0; a[1] = -P.g; a[2] = 0.0;
    st.dt = Q.lens_dt[s]; st.n_done = Q.n_done[s]; st.n_total = Q.n_total[s];
  }
  __device__ void load_vz(const Queue&, unsigned) {}
  __device__ void load_rest(const Queue&, unsigned, LensStep&, bool) {}
  static constexpr bool kDeferLensSetup = false;
};

// ===========================================================================
// FP32 fast path
// ===========================================================================
template <bool kOut, bool kRec>
struct Mol32 {
  float x, y, vx, vy, vz, inv_vz, t;
  float gap0;     // first flight length (from the initial z)
  float margin;
  int rows;
  int32_t id;
  double zc;      // current z, kept only for outputs / recording
  float ax, ay;   // stored acceleration (recording)
  float cx, cy, cvx, cvy;  // rounding errors carried by the lens integration
  RowSink* sink;

  __device__ void row_out() {
    if (kRec) sink->put(x, y, zc, vx, vy, vz, ax, ay, 0.0, t);
  }

  __device__ void init(const Plan& P, const RunDev& R, int64_t i) {
    id = int32_t(i);
    margin = INFINITY;
    rows = 0;
    double z_ic;
    if (R.ic_mode == CTRAJ_IC_DEVICE_DRAW) {
      const Words8 w = molecule_words(R.offset + uint64_t(i), R.key);
      float n0, n1, n2, n3, n4, n5;
      box_muller(w.w[0], w.w[1], n0, n1);
      box_muller(w.w[2], w.w[3], n2, n3);
      box_muller(w.w[4], w.w[5], n4, n5);
      const double* vp = R.vd.p;
      vx = __fmaf_rn(float(vp[1]), n0, float(vp[0]));
      vy = __fmaf_rn(float(vp[3]), n1, float(vp[2]));
      vz = __fmaf_rn(float(vp[5]), n2, float(vp[4]));
      const double* xp = R.xd.p;
      if (R.xd.kind == CTRAJ_DIST_DISC_POSITION) {
        float s, c;
        sincospif(2.0f * u01f(w.w[6]), &s, &c);
        const float rr = __fmul_rn(sqrtf(u01f(w.w[7])), float(xp[0] * 0.5));
        x = __fmul_rn(rr, c);
        y = __fmul_rn(rr, s);
        z_ic = xp[1];
      } else {
        x = __fmul_rn(float(xp[0]), n3);
        y = __fmul_rn(float(xp[1]), n4);
        z_ic = xp[2];
      }
      gap0 = R.gap0f;
    } else {
      const size_t n = size_t(R.n);
      x = float(R.ics[size_t(i)]);
      y = float(R.ics[n + size_t(i)]);
      z_ic = R.ics[2 * n + size_t(i)];
      vx = float(R.ics[3 * n + size_t(i)]);
      vy = float(R.ics[4 * n + size_t(i)]);
      vz = float(R.ics[5 * n + size_t(i)]);
      gap0 = P.n_el > 0 ? float(P.el[0].z0 - z_ic) : 0.0f;
    }
    inv_vz = __frcp_rn(vz);
    t = 0.0f;
    ax = 0.0f;
    ay = -P.gf;
    if (kOut || kRec) zc = z_ic;
    if (kRec) sink->write(x, y, zc, vx, vy, vz, ax, ay, 0.0, t);
  }

  // The device draw of init in two parts, for the front's screening of
  // element 0 (FP32 runs without per-molecule outputs, Gaussian positions):
  // screen_draw: the first Philox call's words, vx, vy, vz and x exactly as
  // init draws them; screen_rest: the second call (y) and the rest of init.
  static constexpr bool kScreenable = !kOut && !kRec;
  __device__ void screen_draw(const RunDev& R, int64_t i) {
    const Philox4 a = philox4x32_10(R.offset + uint64_t(i), 0u, R.key);
    float n0, n1, n2, n3;
    box_muller(a.v[0], a.v[1], n0, n1);
    box_muller(a.v[2], a.v[3], n2, n3);
    const double* vp = R.vd.p;
    vx = __fmaf_rn(float(vp[1]), n0, float(vp[0]));
    vy = __fmaf_rn(float(vp[3]), n1, float(vp[2]));
    vz = __fmaf_rn(float(vp[5]), n2, float(vp[4]));
    x = __fmul_rn(float(R.xd.p[0]), n3);
  }
  __device__ void screen_rest(const Plan& P, const RunDev& R, int64_t i) {
    const Philox4 b = philox4x32_10(R.offset + uint64_t(i), 1u, R.key);
    float n4, n5;
    box_muller(b.v[0], b.v[1], n4, n5);
    y = __fmul_rn(float(R.xd.p[1]), n4);
    id = int32_t(i);
    margin = INFINITY;
    rows = 0;
    gap0 = R.gap0f;
    inv_vz = __frcp_rn(vz);
    t = 0.0f;
    ax = 0.0f;
    ay = -P.gf;
  }
  // True when the walk would stop this molecule (vx, vz, x from screen_draw)
  // at the entrance plane of element 0, a circular or rectangular aperture,
  // whatever its y: after the flight x' = fma(0, h, fma(vx, dt, x)) of the
  // walk, x'^2 > R^2 makes fma(y', y', x'^2) > R^2 for every finite y' (the
  // rounding is monotone), and x' outside (x1, x2) fails the rectangle.  y'
  // is finite when h, vy dt and g h are (y itself is finite, its sigma
  // being so: the caller checks); otherwise the molecule is not screened.
  // The molecule then has the walk's one trajectory row.
  __device__ bool screened_out(const Plan& P, const float gap0f) const {
    const float dt = __fmul_rn(gap0f, __frcp_rn(vz));  // the walk's first flight (fly, element 0)
    const float h = __fmul_rn(__fmul_rn(0.5f, dt), dt);
    if (!(isfinite(h) && fabsf(__fmul_rn(vy, dt)) < 1e30f && fabsf(__fmul_rn(P.gf, h)) < 1e30f)) return false;
    const float xe = __fmaf_rn(0.0f, h, __fmaf_rn(vx, dt, x));
    const float* c = P.ef[0].c;
    return P.el[0].type == CTRAJ_CIRCULAR_APERTURE ? __fmul_rn(xe, xe) > c[0] : !(c[0] < xe && xe < c[1]);
  }

  // ballistic flight of dt with stored acceleration (ax, ay); afterwards a = (0, -g)
  __device__ void flight(float dt, const Plan& P) {
    const float h = __fmul_rn(__fmul_rn(0.5f, dt), dt);
    x = __fmaf_rn(ax, h, __fmaf_rn(vx, dt, x));
    y = __fmaf_rn(ay, h, __fmaf_rn(vy, dt, y));
    vx = __fmaf_rn(ax, dt, vx);
    vy = __fmaf_rn(ay, dt, vy);
    t = __fadd_rn(t, dt);
    ax = 0.0f;
    ay = -P.gf;
    rows += isfinite(t) ? 1 : 0;
  }

  __device__ void fly(const Plan& P, int i, int which) {
    const float gap = which ? P.ef[i].len : (i == 0 ? gap0 : P.ef[i].gap);
    flight(__fmul_rn(gap, inv_vz), P);
    if (kOut || kRec) zc = which ? P.el[i].z1 : P.el[i].z0;
    row_out();
  }

  __device__ void note(float d) {
    if (kOut) margin = fminf(margin, fabsf(d));
  }

  __device__ bool circle_out(const Plan& P, int i) {
    const float r2 = __fmaf_rn(y, y, __fmul_rn(x, x));
    if (kOut) note(__fadd_rn(sqrtf(r2), -P.ef[i].c[1]));
    return r2 > P.ef[i].c[0];
  }
  __device__ bool rect_out(const Plan& P, int i) {
    const float* c = P.ef[i].c;
    if (kOut) { note(x - c[0]); note(x - c[1]); note(y - c[2]); note(y - c[3]); }
    return !((c[0] < x && x < c[1]) && (c[2] < y && y < c[3]));
  }
  __device__ bool plates(const Plan& P, int i) {
    const float x1 = P.ef[i].c[0], x2 = P.ef[i].c[1];
    if (kOut) { note(x - x1); note(x - x2); }
    if (!(x1 < x && x < x2)) return true;
    float dt = __fmul_rn(P.ef[i].len, inv_vz);
    const float xe = __fmaf_rn(vx, dt, x);  // a_x = 0 after a ballistic flight
    if (kOut) { note(xe - x1); note(xe - x2); }
    if (!(x1 < xe && xe < x2)) {
      if (vx < 0.0f) dt = __fdiv_rn(x1 - x, vx);
      else if (vx > 0.0f) dt = __fdiv_rn(x2 - x, vx);
      flight(dt, P);
      if (kOut || kRec) zc += double(dt) * double(vz);
      row_out();
      return true;
    }
    flight(dt, P);
    if (kOut || kRec) zc = P.el[i].z1;
    row_out();
    return false;
  }
  // Honeycomb (meshes.py:98-116) on the float centre table; ef c[0] = R sqrt(3)/2,
  // c[1] = R.
  __device__ bool honeycomb_out(const Plan& P, int i, int& cell) {
    const LensF& L = P.lf[i];
    const float* c = P.ef[i].c;
    if (cell <= 0) {
      float best2, second2;
      cell = mesh_nearest32(L, P.ef[i], x, y, best2, second2);
      if (kOut) note(0.5f * (sqrtf(second2) - sqrtf(best2)));
    }
    const float4 q = __ldg(L.q + cell);
    const float dx = fabsf(x - q.x), dy = fabsf(y - q.y);
    const float lim = __fmaf_rn(-0.57735026919f, dx, c[1]);
    if (kOut) note(fminf(c[0] - dx, 0.8660254038f * (lim - dy)));
    return !(dx < c[0] && dy < lim);
  }
  __device__ bool lens_entrance_out(const Plan& P, int i) { return circle_out(P, i); }

  __device__ double vel_z() const { return double(vz); }

  // kScaled (batched sweeps): the table holds the unscaled polynomial and each
  // molecule brings its configuration's coordinate scale beta and force scale
  // kappa; otherwise both come from L (kappa folded into the table).
  template <int F, bool kStaged, bool kScaled = false>
  __device__ bool lens_step(const LensArgs& L, const float dt, const float hdt, const float c2,
                            const float dt6, const float dt26, const float4* s_tab, unsigned& flags,
                            const float beta = 0.0f, const float kappa = 1.0f) {
    const float g = L.g;
    const float b = kScaled ? beta : L.beta;
    auto force = [&](float px, float py) {
      const float w = wforce<F, kStaged, kScaled>(px, py, L, s_tab, flags, b);
      return kScaled ? __fmul_rn(kappa, w) : w;
    };
    // The (x, y) pairs go through the packed FP32 instructions of sm_100+
    // (FFMA2 / FADD2 / FMUL2): per component the same rounding as the scalar
    // operations, half the instructions.  Increments are formed in full
    // precision, then added once with the carried rounding error (the lens
    // defocuses, so uncompensated rounding of x and v grows to micrometres at
    // the detector).
    const float2 p = make_float2(x, y), v = make_float2(vx, vy);
    const float2 Hdt = make_float2(hdt, hdt), Dt = make_float2(dt, dt), G0 = make_float2(0.0f, -g);
    const float w1 = force(x, y);
    const float2 l1 = __ffma2_rn(make_float2(w1, w1), p, G0);
    const float2 k2 = __ffma2_rn(Hdt, l1, v);
    const float2 p2 = __ffma2_rn(make_float2(c2, c2), v, p);
    const float w2 = force(p2.x, p2.y);
    const float2 l2 = __ffma2_rn(make_float2(w2, w2), p2, G0);
    const float2 k3 = __ffma2_rn(Hdt, l2, v);
    const float2 p3 = __ffma2_rn(Hdt, k2, p);
    const float w3 = force(p3.x, p3.y);
    const float2 l3 = __ffma2_rn(make_float2(w3, w3), p3, G0);
    const float2 p4 = __ffma2_rn(Dt, k3, p);
    const float w4 = force(p4.x, p4.y);
    const float2 l4 = __ffma2_rn(make_float2(w4, w4), p4, G0);
    const float2 sum = __fadd2_rn(__fadd2_rn(l1, l2), l3);
    const float2 dx = __ffma2_rn(make_float2(dt26, dt26), sum, __fmul2_rn(Dt, v));
    const float2 dv = __fmul2_rn(make_float2(dt6, dt6),
                                 __ffma2_rn(make_float2(2.0f, 2.0f), __fadd2_rn(l2, l3), __fadd2_rn(l1, l4)));
    // s += inc with the rounding error carried in c, for both pairs (Fast2Sum:
    // |s| >= |inc + c| holds because one step changes x and v by far less
    // than their size)
    auto neg = [](float2 a) { return make_float2(-a.x, -a.y); };
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
    ax = l1.x;
    ay = l1.y;
    const float r2 = __fmaf_rn(y, y, __fmul_rn(x, x));
    if (kOut) note(__fadd_rn(sqrtf(r2), -L.bore));
    return r2 > L.bore2;
  }

  // Inside the lens t keeps the entrance time and z is not tracked: both
  // follow from the step count (t + n dt, z0 + n dz) instead of being
  // accumulated in float.
  __device__ void lens_begin(const Plan&, int, const LensStep&) { cx = cy = cvx = cvy = 0.0f; }
  __device__ double lens_dz(const ctraj_element& e) const {
    return e.step_mode == CTRAJ_STEP_DT ? dmul(double(vz), e.p[2]) : e.p[1];
  }
  __device__ void lens_row(const Plan& P, int i, const LensStep& s) {
    if (kRec) {
      zc = P.el[i].z0 + double(s.n_done) * lens_dz(P.el[i]);
      sink->put(x, y, zc, vx, vy, vz, ax, ay, 0.0, double(t) + double(s.n_done) * s.dt);
    }
  }
  // After the last step: t from the step count, then the exit snap of
  // (z1 - z0 - N dz) / vz with the stored acceleration l1 unless lost inside.
  __device__ void lens_end(const Plan& P, int i, const LensStep& s, bool lost) {
    t = float(double(t) + double(s.n_done) * s.dt);
    rows += int(s.n_done);
    x = __fadd_rn(x, cx);
    y = __fadd_rn(y, cy);
    vx = __fadd_rn(vx, cvx);
    vy = __fadd_rn(vy, cvy);
    if (kOut || kRec) zc = P.el[i].z0 + double(s.n_done) * lens_dz(P.el[i]);
    if (lost) return;
    flight(float(s.snap), P);
    if (kOut || kRec) zc = P.el[i].z1;
    row_out();
  }

  __device__ void final_row(double* f, int64_t i, int64_t n) const {
    const double vals[10] = {x, y, zc, vx, vy, vz, ax, ay, 0.0, t};
    for (int k = 0; k < 10; ++k) f[size_t(k) * size_t(n) + size_t(i)] = vals[k];
  }
  __device__ void flush_last() {
    if (kRec && !sink->last_written) sink->write(x, y, zc, vx, vy, vz, ax, ay, 0.0, t);
  }

  __device__ void store(const Queue& Q, unsigned s, const LensStep& st) const {
    Q.x[s] = x; Q.y[s] = y; Q.vx[s] = vx; Q.vy[s] = vy; Q.vz[s] = vz; Q.t[s] = t;
    Q.cx[s] = cx; Q.cy[s] = cy; Q.cvx[s] = cvx; Q.cvy[s] = cvy;
    Q.lens_dt[s] = st.dt; Q.snap[s] = float(st.snap);
    Q.n_done[s] = int32_t(st.n_done); Q.n_total[s] = int32_t(st.n_total);
    Q.rows[s] = rows; Q.id[s] = id;
    if (kOut) Q.margin[s] = margin;
  }
  // What the RK4 loop needs; the stored acceleration is not carried (the next
  // RK4 step recomputes it).
  __device__ void load_state(const Queue& Q, unsigned s, const Plan& P, LensStep& st) {
    x = Q.x[s]; y = Q.y[s]; vx = Q.vx[s]; vy = Q.vy[s];
    cx = Q.cx[s]; cy = Q.cy[s]; cvx = Q.cvx[s]; cvy = Q.cvy[s];
    st.dt = Q.lens_dt[s];
    st.n_done = Q.n_done[s]; st.n_total = Q.n_total[s];
    ax = 0.0f;
    ay = -P.gf;
    margin = INFINITY;  // edges seen during this chunk; merged with the queued value below
  }
  __device__ void load_vz(const Queue& Q, unsigned s) { vz = Q.vz[s]; }
  static constexpr bool kDeferLensSetup = true;
  // The rest, read after the RK4 loop so it does not occupy registers during
  // it (the exit-snap time too, unless the setup was just done in this chunk).
  __device__ void load_rest(const Queue& Q, unsigned s, LensStep& st, bool snap_from_queue) {
    vz = Q.vz[s];
    t = Q.t[s];
    if (snap_from_queue) st.snap = double(Q.snap[s]);
    rows = Q.rows[s];
    id = Q.id[s];
    inv_vz = __frcp_rn(vz);
    if (kOut) margin = fminf(margin, float(Q.margin[s]));
  }
};

// ---------------------------------------------------------------------------
// Element walk shared by both precisions (beamline.py:20-38).  Starts at
// element `from`; returns the counter slot of the element the molecule was
// lost on, kLabelDetected when it leaves the beamline, or kQueued when it
// passed the entrance of the lens at element index *lens_at.
// ---------------------------------------------------------------------------
template <class M>
__device__ int walk(M& m, const Plan& P, int from, int* lens_at) {
  for (int i = from; i < P.n_el; ++i) {
    const ctraj_element& e = P.el[i];
    switch (e.type) {
      case CTRAJ_CIRCULAR_APERTURE:
        m.fly(P, i, 0);
        if (m.circle_out(P, i)) return e.label;
        m.fly(P, i, 1);
        if (m.circle_out(P, i)) return e.label;
        break;
      case CTRAJ_RECTANGULAR_APERTURE:
        m.fly(P, i, 0);
        if (m.rect_out(P, i)) return e.label;
        m.fly(P, i, 1);
        if (m.rect_out(P, i)) return e.label;
        break;
      case CTRAJ_FIELD_PLATES:
        m.fly(P, i, 0);
        if (m.plates(P, i)) return e.label;
        break;
      case CTRAJ_HONEYCOMB: {
        int cell = -1;  // None
        m.fly(P, i, 0);
        if (m.honeycomb_out(P, i, cell)) return e.label;
        m.fly(P, i, 1);
        if (m.honeycomb_out(P, i, cell)) return e.label;
        break;
      }
      case CTRAJ_ELECTROSTATIC_LENS:
        m.fly(P, i, 0);
        *lens_at = i;  // also reported for a loss at the entrance test
        if (m.lens_entrance_out(P, i)) return e.label;
        return kQueued;
      default:
        return e.label;
    }
  }
  return kLabelDetected;
}

}  // namespace ctraj
