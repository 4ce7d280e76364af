/*
 * ctraj_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.
 *
 * A scalar FP64 CPU restatement of the reference's propagation path, used only
 * as the checker by tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg.  Nothing in the product links or calls it.
 *
 * It follows the reference operation for operation so that, compiled with
 * -ffp-contract=off, it reproduces the reference's float64 results:
 *
 *   mol_update            molecule.py:26-68 (x + v*dt + a*dt**2/2, v + a*dt,
 *                         t + dt; "if not delta_t" keeps the current state)
 *   circular_aperture     apertures.py:92-115   (dead iff rho > d/2)
 *   rectangular_aperture  apertures.py:165-189  (alive iff x1<x<x2 and y1<y<y2)
 *   field_plates          apertures.py:227-270
 *   lens                  electrostatic_lens.py:48-118 (reference RK4 with the
 *                         stage-2 point x + dt*k1, exit snap with a = l1)
 *   lens_force            electrostatic_lens.py:168-227 with the a_interp of
 *                         the table kind:
 *                           RADIAL_LINEAR  scipy interp1d._call_linear, bounds
 *                                          error above the last knot
 *                           STARK_SPLINE   a_r(r) = -(W'(E) * dE/dr) / m with
 *                                          E = alpha r^n and W' the scipy PPoly
 *                                          derivative (nu = 1) evaluation order
 *   honeycomb             meshes.py:85-117 (argmin over all cell centres, re-done
 *                         while the cell index is 0 -- `if not idx`; hexagon
 *                         interior of the RegularPolygon of meshes.py:71-78)
 *   propagate             beamline.py:20-38 (walk, early exit, "Detected")
 *   rows                  Trajectory.update / drop_nans (molecule.py:133-167):
 *                         the step count is the number of finite-t rows - 1
 *
 * Parity pin: tests/golden/make_golden.py runs the reference itself on
 * injected initial conditions and stores its outputs; tests/test_oracle.py
 * checks this file against them.  One deliberate difference: numpy's scalar
 * ``delta_t**2`` on x86-64 goes through a SIMD pow that rounds about 0.08 % of
 * squares one ulp away from the correctly rounded x*x; this file uses x*x, so
 * fixture comparisons allow a few ulp.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "../include/ctraj.h"

#define LABEL_DETECTED (-1)

typedef struct {
  double x[3], v[3], a[3], t;
} row_t;

typedef struct {
  row_t s;             /* current (last stored) trajectory row */
  int alive;
  int label;           /* counter slot, LABEL_DETECTED when alive at the end */
  int64_t rows;        /* finite-t rows stored after the initial one */
  int64_t lens_steps;
  double margin;       /* smallest |edge distance| seen by a hit test */
  int err;             /* CTRAJ_ERANGE / CTRAJ_ESTEPS when the reference would raise */
  /* optional recording of every stored row */
  row_t* rec;
  int64_t rec_max;
  int64_t rec_n;
} mol_t;

typedef struct {
  const ctraj_element* el;
  int n_el;
  const ctraj_force_table* tab;
  int n_tab;
  double g;
} beam_t;

static void push_row(mol_t* m, const double x[3], const double v[3],
                     const double a[3], double t) {
  for (int k = 0; k < 3; k++) {
    m->s.x[k] = x[k];
    m->s.v[k] = v[k];
    m->s.a[k] = a[k];
  }
  m->s.t = t;
  if (isfinite(t)) m->rows++;
  if (m->rec) {
    if (m->rec_n < m->rec_max) m->rec[m->rec_n] = m->s;
    m->rec_n++;
  }
}

static void note_margin(mol_t* m, double d) {
  d = fabs(d);
  if (d < m->margin) m->margin = d;
}

/* Molecule.update_trajectory(delta_t, a=(0,-g,0)), molecule.py:58-68 */
static void mol_update(mol_t* m, double dt, double g) {
  double x[3], v[3];
  const double a_new[3] = {0.0, -g, 0.0};
  if (dt == 0.0) { /* `if not delta_t` returns the current state (:31, :41) */
    for (int k = 0; k < 3; k++) {
      x[k] = m->s.x[k];
      v[k] = m->s.v[k];
    }
  } else {
    double dt2 = dt * dt;
    for (int k = 0; k < 3; k++) {
      x[k] = (m->s.x[k] + m->s.v[k] * dt) + (m->s.a[k] * dt2) / 2.0;
      v[k] = m->s.v[k] + m->s.a[k] * dt;
    }
  }
  push_row(m, x, v, a_new, m->s.t + dt);
}

static double rho_of(const double x[3]) { return sqrt(x[0] * x[0] + x[1] * x[1]); }

static void kill(mol_t* m, int label) {
  m->alive = 0;
  m->label = label;
}

/* CircularAperture.propagate_through, apertures.py:92-115 */
static void circular_aperture(mol_t* m, const ctraj_element* e, double g) {
  const double zs[2] = {e->z0, e->z1};
  for (int i = 0; i < 2; i++) {
    double dt = (zs[i] - m->s.x[2]) / m->s.v[2];
    mol_update(m, dt, g);
    double rho = rho_of(m->s.x);
    note_margin(m, rho - e->p[0] / 2.0);
    if (rho > e->p[0] / 2.0) {
      kill(m, e->label);
      return;
    }
  }
}

/* RectangularAperture.propagate_through, apertures.py:165-189 */
static void rectangular_aperture(mol_t* m, const ctraj_element* e, double g) {
  const double zs[2] = {e->z0, e->z1};
  const double x1 = e->p[0], x2 = e->p[1], y1 = e->p[2], y2 = e->p[3];
  for (int i = 0; i < 2; i++) {
    double dt = (zs[i] - m->s.x[2]) / m->s.v[2];
    mol_update(m, dt, g);
    const double x = m->s.x[0], y = m->s.x[1];
    note_margin(m, x - x1);
    note_margin(m, x - x2);
    note_margin(m, y - y1);
    note_margin(m, y - y2);
    if (!((x1 < x && x < x2) && (y1 < y && y < y2))) {
      kill(m, e->label);
      return;
    }
  }
}

/* FieldPlates.propagate_through, apertures.py:227-270 */
static void field_plates(mol_t* m, const ctraj_element* e, double g) {
  const double x1 = e->p[0], x2 = e->p[1];
  double dt = (e->z0 - m->s.x[2]) / m->s.v[2];
  mol_update(m, dt, g);
  note_margin(m, m->s.x[0] - x1);
  note_margin(m, m->s.x[0] - x2);
  if (!(x1 < m->s.x[0] && m->s.x[0] < x2)) {
    kill(m, e->label);
    return;
  }
  dt = (e->z1 - m->s.x[2]) / m->s.v[2];
  /* molecule.x(delta_t) without storing (:250) */
  double xe;
  if (dt == 0.0)
    xe = m->s.x[0];
  else
    xe = (m->s.x[0] + m->s.v[0] * dt) + (m->s.a[0] * (dt * dt)) / 2.0;
  note_margin(m, xe - x1);
  note_margin(m, xe - x2);
  if (!(x1 < xe && xe < x2)) {
    /* flight to the plate the molecule moves toward; vx == 0 keeps dt (:255-259) */
    if (m->s.v[0] < 0)
      dt = (x1 - m->s.x[0]) / m->s.v[0];
    else if (m->s.v[0] > 0)
      dt = (x2 - m->s.x[0]) / m->s.v[0];
    mol_update(m, dt, g);
    kill(m, e->label);
    return;
  }
  mol_update(m, dt, g);
}

/* scipy PPoly.__call__(E, nu=1) for one point: interval with knots[i] <= E <
 * knots[i+1] (extrapolating the end pieces), then the nu = 1 evaluation order
 * of scipy.interpolate._ppoly.evaluate_poly1. */
static double spline_deriv(const ctraj_force_table* t, double E, int* range) {
  const int n = t->n_knots;
  const double* xk = t->knots;
  int i;
  if (isnan(E)) return NAN;
  if (E < xk[0]) {
    i = 0;
    *range = 1;
  } else if (E >= xk[n - 1]) {
    i = n - 2;
    if (E > xk[n - 1]) *range = 1;
  } else {
    double h = (xk[n - 1] - xk[0]) / (double)(n - 1);
    i = (int)floor((E - xk[0]) / h);
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    while (i > 0 && E < xk[i]) i--;
    while (i < n - 2 && E >= xk[i + 1]) i++;
  }
  const double* c = t->coef + 4 * (size_t)i;
  double s = E - xk[i];
  double res = 0.0;
  res = res + (c[2] * 1.0) * 1.0;
  res = res + (c[1] * s) * 2.0;
  res = res + (c[0] * (s * s)) * 3.0;
  return res;
}

/* scipy interp1d(kind='linear', bounds_error=True)(r).  For float64 1-D data
 * scipy delegates to numpy.interp (interp1d._call_linear_np), whose kernel is:
 * j = last knot <= r; r == knots[j] or j == n-1 -> values[j]; else
 * slope = (y[j+1]-y[j]) / (x[j+1]-x[j]); slope*(r - x[j]) + y[j]. */
static double radial_linear(const ctraj_force_table* t, double r, int* err) {
  const int n = t->n_knots;
  const double* xk = t->knots;
  const double* yk = t->values;
  if (r < xk[0] || r > xk[n - 1]) { /* interp1d._check_bounds raises */
    *err = 1;
    return NAN;
  }
  if (isnan(r)) return r;
  double h = (xk[n - 1] - xk[0]) / (double)(n - 1);
  int j = (int)floor((r - xk[0]) / h);
  if (j < 0) j = 0;
  if (j > n - 1) j = n - 1;
  while (j > 0 && xk[j] > r) j--;
  while (j < n - 1 && xk[j + 1] <= r) j++;
  if (j == n - 1 || xk[j] == r) return yk[j];
  const double slope = (yk[j + 1] - yk[j]) / (xk[j + 1] - xk[j]);
  return slope * (r - xk[j]) + yk[j];
}

/* ElectrostaticLens.lens_acceleration, electrostatic_lens.py:215-227 */
static void lens_force(const beam_t* b, const ctraj_element* e, const double x[3],
                       double a[3], mol_t* m, int* range_count) {
  const ctraj_force_table* t = &b->tab[e->table];
  const double r = rho_of(x);
  double a_r;
  if (t->kind == CTRAJ_TABLE_RADIAL_LINEAR) {
    int err = 0;
    a_r = radial_linear(t, r, &err);
    if (err) m->err = CTRAJ_ERANGE;
  } else {
    const double alpha = e->p[6], mass = e->p[5];
    int range = 0;
    if (e->field_order == 1) {
      double E = alpha * r;
      a_r = -(spline_deriv(t, E, &range) * alpha) / mass;
    } else {
      double E = alpha * (r * r);
      a_r = -(spline_deriv(t, E, &range) * (2.0 * alpha * r)) / mass;
    }
    *range_count += range;
  }
  a[0] = 0.0;
  a[1] = 0.0;
  a[2] = 0.0;
  if (r != 0) {
    a[0] = a_r * x[0] / r;
    a[1] = a_r * x[1] / r;
    a[2] = 0;
  }
  a[1] -= b->g;
}

/* ElectrostaticLens.propagate_through + propagate_inside_lens, :48-118 */
static void lens(mol_t* m, const beam_t* b, const ctraj_element* e, int* range_count) {
  const double d = e->p[0];
  double dt = (e->z0 - m->s.x[2]) / m->s.v[2];
  mol_update(m, dt, b->g);
  double rho = rho_of(m->s.x);
  note_margin(m, rho - d / 2.0);
  if (rho > d / 2.0) {
    kill(m, e->label);
    return;
  }
  const double L = e->p[7];
  double dz = e->step_mode == CTRAJ_STEP_DT ? m->s.v[2] * e->p[2] : e->p[1];
  const double nf = rint(L / dz);
  if (!isfinite(nf) || fabs(nf) > (double)CTRAJ_MAX_LENS_STEPS) {
    m->err = CTRAJ_ESTEPS;
    kill(m, e->label_inside);
    return;
  }
  const int64_t n_steps = (int64_t)nf;
  dt = dz / m->s.v[2];
  const int classic = e->scheme == CTRAJ_RK4_CLASSIC;
  for (int64_t i = 0; i < n_steps; i++) {
    double x[3], k1[3], l1[3], k2[3], l2[3], k3[3], l3[3], k4[3], l4[3], p[3];
    for (int k = 0; k < 3; k++) {
      x[k] = m->s.x[k];
      k1[k] = m->s.v[k];
    }
    lens_force(b, e, x, l1, m, range_count);
    for (int k = 0; k < 3; k++) {
      k2[k] = k1[k] + dt * l1[k] / 2;
      p[k] = classic ? x[k] + dt * k1[k] / 2 : x[k] + dt * k1[k];
    }
    lens_force(b, e, p, l2, m, range_count);
    for (int k = 0; k < 3; k++) {
      k3[k] = k1[k] + dt * l2[k] / 2;
      p[k] = x[k] + dt * k2[k] / 2;
    }
    lens_force(b, e, p, l3, m, range_count);
    for (int k = 0; k < 3; k++) {
      k4[k] = k1[k] + dt * l3[k];
      p[k] = classic ? x[k] + dt * k3[k] : x[k] + dt * k3[k];
    }
    lens_force(b, e, p, l4, m, range_count);
    double xn[3], vn[3];
    for (int k = 0; k < 3; k++) {
      xn[k] = x[k] + dt * (k1[k] + 2 * k2[k] + 2 * k3[k] + k4[k]) / 6;
      vn[k] = k1[k] + dt * (l1[k] + 2 * l2[k] + 2 * l3[k] + l4[k]) / 6;
    }
    push_row(m, xn, vn, l1, m->s.t + dt);
    m->lens_steps++;
    if (m->err) { /* the reference raised inside this step */
      kill(m, e->label_inside);
      return;
    }
    rho = rho_of(m->s.x);
    note_margin(m, rho - d / 2.0);
    if (rho > d / 2.0) {
      kill(m, e->label_inside);
      return;
    }
  }
  dt = (e->z1 - m->s.x[2]) / m->s.v[2];
  mol_update(m, dt, b->g);
}

/* Honeycomb.propagate_through, meshes.py:87-117: flight to z0 and z1; at each
 * plane the molecule must lie inside the hexagon of "its" cell, the cell with
 * the nearest centre found at z0 -- and again at z1 when that cell has index
 * 0, because the reference tests `if not idx:` (:104) and 0 is falsy.  The
 * distances are numpy's sqrt((px - xc)**2 + (py - yc)**2) (:105-107), the first
 * minimum wins (argmin); the hexagon is matplotlib's RegularPolygon((xc, yc),
 * 6, radius=R) with a vertex on +y (:71-78), interior: |dx| < R sqrt(3)/2 and
 * |dy| < R - |dx|/sqrt(3).  Edge margins: the hexagon's sides and half the gap
 * between the nearest and second-nearest centre. */
static void honeycomb(mol_t* m, const beam_t* b, const ctraj_element* e) {
  const ctraj_force_table* t = &b->tab[e->table];
  const double zs[2] = {e->z0, e->z1};
  const double s3 = sqrt(3.0), R = e->p[0];
  int idx = -1; /* None */
  for (int i = 0; i < 2; i++) {
    double dt = (zs[i] - m->s.x[2]) / m->s.v[2];
    mol_update(m, dt, b->g);
    const double px = m->s.x[0], py = m->s.x[1];
    if (idx <= 0) {
      double best = INFINITY, second = INFINITY;
      for (int k = 0; k < t->n_knots; k++) {
        const double dx = px - t->knots[k], dy = py - t->values[k];
        const double d = sqrt(dx * dx + dy * dy);
        if (d < best) {
          second = best;
          best = d;
          idx = k;
        } else if (d < second) {
          second = d;
        }
      }
      if (idx < 0) idx = 0; /* no finite distance: argmin of all-NaN is 0 */
      note_margin(m, (second - best) / 2.0);
    }
    const double dx = fabs(px - t->knots[idx]), dy = fabs(py - t->values[idx]);
    const double side = R * s3 / 2.0 - dx, slant = (R - dx / s3 - dy) * (s3 / 2.0);
    note_margin(m, side < slant ? side : slant);
    if (!(dx < R * s3 / 2.0 && dy < R - dx / s3)) {
      kill(m, e->label);
      return;
    }
  }
}

/* Molecule.init_trajectory + Beamline.propagate_through */
static void propagate(const beam_t* b, const double ic[6], mol_t* m, int* range_count) {
  m->alive = 1;
  m->label = LABEL_DETECTED;
  m->rows = 0;
  m->lens_steps = 0;
  m->margin = INFINITY;
  m->err = 0;
  const double x0[3] = {ic[0], ic[1], ic[2]};
  const double v0[3] = {ic[3], ic[4], ic[5]};
  const double a0[3] = {0.0, -b->g, 0.0};
  /* the initial row is not a step */
  push_row(m, x0, v0, a0, 0.0);
  m->rows = 0;
  for (int i = 0; i < b->n_el && m->alive; i++) {
    const ctraj_element* e = &b->el[i];
    switch (e->type) {
      case CTRAJ_CIRCULAR_APERTURE: circular_aperture(m, e, b->g); break;
      case CTRAJ_RECTANGULAR_APERTURE: rectangular_aperture(m, e, b->g); break;
      case CTRAJ_FIELD_PLATES: field_plates(m, e, b->g); break;
      case CTRAJ_ELECTROSTATIC_LENS: lens(m, b, e, range_count); break;
      case CTRAJ_HONEYCOMB: honeycomb(m, b, e); break;
      default: m->err = CTRAJ_EINVAL; m->alive = 0; break;
    }
  }
}

/* ---- public oracle entry points (ctypes) ---------------------------------- */

typedef struct {
  beam_t b;
  const double* ics; /* (6, n) */
  int64_t n, lo, hi;
  int32_t* label;
  double* fin;       /* (10, n) */
  int32_t* rows;
  double* margin;
  int64_t* counts;   /* n_labels + 1, per thread */
  int n_labels;
  int64_t steps, lens_steps, edge_band, range_count, errors;
  int first_err;
} job_t;

static void* run_job(void* arg) {
  job_t* j = (job_t*)arg;
  for (int64_t i = j->lo; i < j->hi; i++) {
    double ic[6];
    for (int k = 0; k < 6; k++) ic[k] = j->ics[(size_t)k * j->n + i];
    mol_t m;
    memset(&m, 0, sizeof m);
    int range = 0;
    propagate(&j->b, ic, &m, &range);
    j->range_count += range;
    if (m.err) {
      j->errors++;
      if (!j->first_err) j->first_err = m.err;
    }
    j->steps += m.rows;
    j->lens_steps += m.lens_steps;
    if (m.margin < 1e-6) j->edge_band++;
    if (j->counts) {
      int slot = m.label < 0 ? j->n_labels : m.label;
      j->counts[slot]++;
    }
    if (j->label) j->label[i] = m.label;
    if (j->rows) j->rows[i] = (int32_t)m.rows;
    if (j->margin) j->margin[i] = m.margin;
    if (j->fin) {
      const double* src[10] = {&m.s.x[0], &m.s.x[1], &m.s.x[2], &m.s.v[0], &m.s.v[1],
                               &m.s.v[2], &m.s.a[0], &m.s.a[1], &m.s.a[2], &m.s.t};
      for (int k = 0; k < 10; k++) j->fin[(size_t)k * j->n + i] = *src[k];
    }
  }
  return NULL;
}

/*
 * Propagate n molecules with initial conditions ics (6, n) on `threads` host
 * threads.  counts has n_labels + 1 slots (last = "Detected").  stats[0..4] =
 * molecule steps, lens steps, edge-band molecules, out-of-range lookups,
 * molecules on which the reference would have raised.  Returns CTRAJ_OK or
 * the first error status a molecule hit.
 */
int ctraj_oracle_run(const ctraj_element* el, int n_el, const ctraj_force_table* tab,
                     int n_tab, double g, const double* ics, int64_t n, int n_labels,
                     int threads, int32_t* label, double* fin, int32_t* rows,
                     double* margin, int64_t* counts, int64_t* stats) {
  if (threads < 1) threads = 1;
  if (threads > 256) threads = 256;
  job_t* jobs = (job_t*)calloc((size_t)threads, sizeof(job_t));
  int64_t* tc = (int64_t*)calloc((size_t)threads * (size_t)(n_labels + 1), sizeof(int64_t));
  pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
  if (!jobs || !tc || !th) {
    free(jobs); free(tc); free(th);
    return CTRAJ_ENOMEM;
  }
  for (int t = 0; t < threads; t++) {
    job_t* j = &jobs[t];
    j->b.el = el; j->b.n_el = n_el; j->b.tab = tab; j->b.n_tab = n_tab; j->b.g = g;
    j->ics = ics; j->n = n;
    j->lo = n * t / threads;
    j->hi = n * (t + 1) / threads;
    j->label = label; j->fin = fin; j->rows = rows; j->margin = margin;
    j->counts = tc + (size_t)t * (n_labels + 1);
    j->n_labels = n_labels;
  }
  for (int t = 1; t < threads; t++) pthread_create(&th[t], NULL, run_job, &jobs[t]);
  run_job(&jobs[0]);
  for (int t = 1; t < threads; t++) pthread_join(th[t], NULL);
  int status = CTRAJ_OK;
  int64_t s[5] = {0, 0, 0, 0, 0};
  for (int t = 0; t < threads; t++) {
    job_t* j = &jobs[t];
    s[0] += j->steps; s[1] += j->lens_steps; s[2] += j->edge_band;
    s[3] += j->range_count; s[4] += j->errors;
    if (status == CTRAJ_OK && j->first_err) status = j->first_err;
    if (counts)
      for (int k = 0; k <= n_labels; k++) counts[k] += j->counts[k];
  }
  if (stats) memcpy(stats, s, sizeof s);
  free(jobs); free(tc); free(th);
  return status;
}

/*
 * Full trajectory of one molecule: every stored row (x, v, a, t as 10 doubles)
 * including the initial one, up to max_rows.  Returns the number of rows the
 * molecule produced (may exceed max_rows), *label_out its counter slot.
 */
int64_t ctraj_oracle_trace(const ctraj_element* el, int n_el, const ctraj_force_table* tab,
                           int n_tab, double g, const double ic[6], double* out_rows,
                           int64_t max_rows, int32_t* label_out) {
  beam_t b = {el, n_el, tab, n_tab, g};
  mol_t m;
  memset(&m, 0, sizeof m);
  m.rec = (row_t*)out_rows;
  m.rec_max = max_rows;
  int range = 0;
  propagate(&b, ic, &m, &range);
  if (label_out) *label_out = m.label;
  return m.rec_n;
}

int ctraj_oracle_abi(void) { return CTRAJ_ABI_VERSION; }
