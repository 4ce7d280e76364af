// libctraj.so: C ABI of the GB300 trajectory engine (declared in include/ctraj.h):
// contexts, runs, pipelined batches, ring recording, trajectory replay.  The
// batched sweep (sweep.cu), the soft transmission (soft.cu), the
// allocation-free run (noalloc.cu) and the kernel families (k_front.cu,
// k_chunk.cu, k_persist.cu) are translation units of their own.
//
// A context owns one CUDA stream (or borrows the caller's), the device copies
// of the beamline's force tables, the FP32 lens tables derived from them, and
// grow-only work buffers (lens queues, injected initial conditions,
// per-molecule outputs).  ctraj_run enqueues k_front and the chunked lens
// kernels and copies the per-label counts back; nothing is allocated on a
// repeated run of the same or a smaller size.
#include <mutex>
#include <system_error>
#include <thread>
#include <type_traits>

#include "engine.h"
#include "kernels.cuh"

namespace ctraj {

thread_local std::string g_error;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_error = buf;
  return code;
}

// Queue layout inside one buffer of capacity cap (SoA, each array 256-byte
// aligned so a warp's 32 consecutive entries are whole 128-byte lines).
// Returns the bytes used; with b == nullptr only sizes the layout.
size_t layout_queue(const DevBuf* b, size_t cap, int precision, unsigned* ctl, Queue* q,
                    bool with_cfg) {
  Queue tmp{};
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += align256(bytes);
    return o;
  };
  auto f = [&](float** p) { size_t o = take(cap * 4); if (b) *p = b->as<float>(o); };
  auto d = [&](double** p) { size_t o = take(cap * 8); if (b) *p = b->as<double>(o); };
  auto i = [&](int32_t** p) { size_t o = take(cap * 4); if (b) *p = b->as<int32_t>(o); };
  if (precision == 32) {
    f(&tmp.x); f(&tmp.y); f(&tmp.vx); f(&tmp.vy); f(&tmp.vz); f(&tmp.t);
    f(&tmp.cx); f(&tmp.cy); f(&tmp.cvx); f(&tmp.cvy); f(&tmp.snap);
  } else {
    d(&tmp.dx); d(&tmp.dy); d(&tmp.dz); d(&tmp.dvx); d(&tmp.dvy); d(&tmp.dvz); d(&tmp.dt);
  }
  d(&tmp.lens_dt);
  d(&tmp.margin);
  i(&tmp.rows); i(&tmp.id); i(&tmp.n_done); i(&tmp.n_total);
  if (with_cfg) i(&tmp.cfg);
  tmp.count = ctl;
  tmp.max_steps = ctl ? ctl + 1 : nullptr;
  tmp.head = ctl ? ctl + 2 : nullptr;
  if (q) *q = tmp;
  return off;
}

size_t queue_bytes(size_t cap, int precision, bool with_cfg) {
  return layout_queue(nullptr, cap, precision, nullptr, nullptr, with_cfg);
}

bool stark_linear(int kind, int n_knots, const double* knots, const double* coef, const ctraj_element& e) {
  if (kind != CTRAJ_TABLE_STARK_SPLINE || e.field_order != 2 || n_knots < 2) return false;
  const int n_int = n_knots - 1;
  if (2 * n_int > kMaxStagedLinear) return false;
  const double h = (knots[n_int] - knots[0]) / double(n_int), alpha = e.p[6];
  const double rc = 0.5 * e.p[0] * kLinearCover;
  if (!(alpha >= 0.0) || !(knots[0] <= 0.0) || !(alpha * rc * rc <= knots[n_int])) return false;
  double cmax = 0.0, wmax = 0.0;
  for (int j = 0; j < n_int; ++j) {
    const double* cj = coef + size_t(j) * 4;
    const double a = cj[2], b = 2.0 * cj[1] * h, c = 3.0 * cj[0] * h * h;
    cmax = std::max(cmax, std::fabs(c));
    wmax = std::max(wmax, std::max(std::fabs(a), std::fabs(a + b + c)));
  }
  return std::isfinite(cmax) && cmax / double(4 * kLinearPieces * kLinearPieces) <= kLinearTolerance * wmax;
}

// Float4 `half` (0 or 1) of a kForceStark2Lin knot interval: the quadratic
// a + b u + c u^2 (u in [0, 1]) as linear pieces over the quarters, each
// (w at the piece's start, its rise across it), two pieces per float4.
float4 stark_pieces(double a, double b, double c, int half) {
  auto w = [&](int k) { const double u = 0.25 * k; return a + u * (b + u * c); };
  const int k = 2 * half;
  return make_float4(float(w(k)), float(w(k + 1) - w(k)), float(w(k + 1)), float(w(k + 2) - w(k + 1)));
}

int lens_force_kind(const ctraj_context* c, const ctraj_element& e) {
  const HostTable& t = c->tables[e.table];
  if (t.kind == CTRAJ_TABLE_RADIAL_LINEAR) return kForceRadial;
  if (stark_linear(t.kind, t.n, t.knots.data(), t.coef.data(), e)) return kForceStark2Lin;
  return e.field_order == 1 ? kForceStark1 : kForceStark2;
}

// FP32 lens tables: coefficients of the per-interval polynomial in the local
// coordinate u (0..1), pre-multiplied by the lens's force prefactor.
int build_lens_tables(ctraj_context* c) {
  const int n_el = int(c->elements.size());
  c->lens_offset.assign(n_el, 0);
  c->lens_n_int.assign(n_el, 0);
  c->lens_n_smem.assign(n_el, 0);
  c->lens_outward.assign(n_el, 0);
  std::vector<float4> host;
  for (int i = 0; i < n_el; ++i) {
    const ctraj_element& e = c->elements[i];
    if (e.type == CTRAJ_HONEYCOMB) {  // cell centres (x, y, 0, 0)
      const HostTable& t = c->tables[e.table];
      c->lens_offset[i] = host.size();
      c->lens_n_int[i] = t.n;
      for (int k = 0; k < t.n; ++k) host.push_back(make_float4(float(t.knots[k]), float(t.values[k]), 0.f, 0.f));
      continue;
    }
    if (e.type != CTRAJ_ELECTROSTATIC_LENS) continue;
    const HostTable& t = c->tables[e.table];
    const double x0 = t.knots[0], h = (t.knots[t.n - 1] - t.knots[0]) / double(t.n - 1);
    const int n_int = t.n - 1;
    const bool lin = lens_force_kind(c, e) == kForceStark2Lin;
    c->lens_offset[i] = host.size();
    c->lens_n_int[i] = lin ? 2 * n_int : n_int;  // float4 entries
    (void)x0;
    if (t.kind == CTRAJ_TABLE_RADIAL_LINEAR) {
      for (int j = 0; j < n_int; ++j)
        host.push_back(make_float4(float(t.values[j]), float(t.values[j + 1] - t.values[j]), 0.f, 0.f));
    } else {
      const double alpha = e.p[6], mass = e.p[5];
      const double kappa = e.field_order == 1 ? alpha / mass : 2.0 * alpha / mass;
      for (int j = 0; j < n_int; ++j) {
        const double* cj = &t.coef[size_t(j) * 4];
        const double qa = -kappa * cj[2], qb = -kappa * 2.0 * cj[1] * h, qc = -kappa * 3.0 * cj[0] * h * h;
        if (lin) {
          host.push_back(stark_pieces(qa, qb, qc, 0));
          host.push_back(stark_pieces(qa, qb, qc, 1));
        } else {
          host.push_back(make_float4(float(qa), float(qb), float(qc), 0.f));
        }
      }
    }
    // a Stark table whose w >= 0 at every piece's ends (the linear form) or
    // interval's ends (the quadratic), up to 1e-5 of its largest |w| (the
    // spline's wiggle at |E| = 0), pushes molecules outward: the lens
    // defocuses, which the entrant order uses
    if (t.kind != CTRAJ_TABLE_RADIAL_LINEAR) {
      float wmax = 0.f;
      for (size_t k = c->lens_offset[i]; k < host.size(); ++k)
        wmax = std::max(wmax, std::max(std::fabs(host[k].x), std::fabs(host[k].z)));
      const float tol = -1e-5f * wmax;
      bool out = true;
      for (size_t k = c->lens_offset[i]; k < host.size() && out; ++k) {
        const float4 q = host[k];
        out = lin ? (q.x >= tol && q.x + q.y >= tol && q.z >= tol && q.z + q.w >= tol)
                  : (q.x >= tol && q.x + q.y + q.z >= tol);
      }
      c->lens_outward[i] = out ? 1 : 0;
    }
    // the whole table goes to shared memory when it takes at most 96 KiB
    // (128 KiB in the linear form)
    const int entries = c->lens_n_int[i];
    c->lens_n_smem[i] = entries <= (lin ? kMaxStagedLinear : kMaxStagedIntervals) ? entries : 0;
  }
  if (!host.empty()) {
    int st = c->lens_tables.ensure(host.size() * sizeof(float4));
    if (st) return st;
    CT_CUDA(cudaMemcpyAsync(c->lens_tables.p, host.data(), host.size() * sizeof(float4),
                            cudaMemcpyHostToDevice, c->stream));
  }
  c->lens_tables_dirty = false;
  return CTRAJ_OK;
}

// FP32 constants of a honeycomb: hexagon half width R sqrt(3)/2, R, and the
// inverse row and cell pitches that place the nearest-centre window.
void honeycomb_constants(const ctraj_element& e, ElemF& f) {
  f.c[0] = float(e.p[0] * std::sqrt(3.0) / 2.0);
  f.c[1] = float(e.p[0]);
  f.c[2] = float(e.p[2]);
  f.c[3] = float(e.p[3]);
}

// A honeycomb's mesh table: kind MESH, whole rows of p[1] cells.
int check_honeycomb(const ctraj_element& e, int i, int kind, int n) {
  if (kind != CTRAJ_TABLE_MESH) return fail(CTRAJ_EINVAL, "honeycomb element %d: table %d is not a mesh table", i, e.table);
  const double nx = e.p[1];
  if (!(nx >= 1.0) || nx != std::floor(nx) || nx > double(n) || n % int(nx) != 0)
    return fail(CTRAJ_EINVAL, "honeycomb element %d: %d cells do not form rows of p[1] = %g cells", i, n, nx);
  if (!std::isfinite(e.p[2]) || !std::isfinite(e.p[3]) || !(e.p[0] >= 0.0))
    return fail(CTRAJ_EINVAL, "honeycomb element %d: bad radius or pitches", i);
  return CTRAJ_OK;
}

int build_plan(ctraj_context* c, const ctraj_run_args* a, Plan& P) {
  std::memset(&P, 0, sizeof P);
  const int n_el = int(c->elements.size());
  P.n_el = n_el;
  P.n_labels = c->n_labels;
  P.first_lens = n_el;
  P.g = a->g;
  P.gf = float(a->g);
  for (int i = 0; i < n_el; ++i) {
    const ctraj_element& e = c->elements[i];
    P.el[i] = e;
    ElemF& f = P.ef[i];
    f.gap = i > 0 ? float(e.z0 - c->elements[i - 1].z1) : 0.f;
    f.len = float(e.z1 - e.z0);
    switch (e.type) {
      case CTRAJ_CIRCULAR_APERTURE:
      case CTRAJ_ELECTROSTATIC_LENS: {
        const double h = e.p[0] * 0.5;
        f.c[0] = float(h * h);
        f.c[1] = float(h);
        break;
      }
      case CTRAJ_RECTANGULAR_APERTURE:
        for (int k = 0; k < 4; ++k) f.c[k] = float(e.p[k]);
        break;
      case CTRAJ_FIELD_PLATES:
        f.c[0] = float(e.p[0]);
        f.c[1] = float(e.p[1]);
        break;
      case CTRAJ_HONEYCOMB:
        honeycomb_constants(e, f);
        break;
    }
    if (e.type == CTRAJ_HONEYCOMB) {
      LensF& L = P.lf[i];
      L.q = c->lens_tables.as<float4>(c->lens_offset[i] * sizeof(float4));
      L.n_int = c->lens_n_int[i];
      L.cols = int(e.p[1]);
    }
    if (e.type == CTRAJ_ELECTROSTATIC_LENS) {
      if (P.first_lens == n_el) P.first_lens = i;
      const HostTable& t = c->tables[e.table];
      LensF& L = P.lf[i];
      const double x0 = t.knots[0], h = (t.knots[t.n - 1] - t.knots[0]) / double(t.n - 1);
      L.q = c->lens_tables.as<float4>(c->lens_offset[i] * sizeof(float4));
      L.n_int = c->lens_n_int[i];
      L.n_smem = c->lens_n_smem[i];
      L.outward = c->lens_outward[i];
      L.force = lens_force_kind(c, e);
      if (t.kind == CTRAJ_TABLE_RADIAL_LINEAR) {
        L.beta = float(1.0 / h);
        L.s0 = float(x0 / h);
        L.r_max = float(t.knots[t.n - 1]);
      } else {
        const double scale = L.force == kForceStark2Lin ? double(kLinearPieces) : 1.0;  // pieces
        L.beta = float(scale * e.p[6] / h);
        L.s0 = float(scale * x0 / h);
        L.r_max = INFINITY;
      }
    }
  }
  for (int k = 0; k < CTRAJ_MAX_TABLES; ++k) {
    const HostTable& t = c->tables[k];
    if (!t.n) continue;
    TableD& d = P.td[k];
    d.kind = t.kind;
    d.n = t.n;
    d.x0 = t.knots[0];
    d.h = (t.knots[t.n - 1] - t.knots[0]) / double(t.n - 1);
    d.knots = t.dev.as<double>(0);
    d.coef = t.coef.empty() ? nullptr : t.dev.as<double>(align256(t.n * 8));
    d.values = t.values.empty() ? nullptr : t.dev.as<double>(align256(t.n * 8));
  }
  return CTRAJ_OK;
}

int check_beamline(const ctraj_context* c) {
  for (size_t i = 0; i < c->elements.size(); ++i) {
    const ctraj_element& e = c->elements[i];
    if (e.type == CTRAJ_ELECTROSTATIC_LENS) {
      if (e.table < 0 || e.table >= CTRAJ_MAX_TABLES || !c->tables[e.table].n)
        return fail(CTRAJ_ESTATE, "lens element %zu uses force table %d, which is not set", i, e.table);
      const HostTable& t = c->tables[e.table];
      if (t.kind == CTRAJ_TABLE_MESH) return fail(CTRAJ_EINVAL, "lens element %zu: table %d is a mesh table", i, e.table);
      if (t.kind == CTRAJ_TABLE_STARK_SPLINE && e.field_order != 1 && e.field_order != 2)
        return fail(CTRAJ_EINVAL, "lens element %zu: field_order must be 1 or 2", i);
    } else if (e.type == CTRAJ_HONEYCOMB) {
      if (e.table < 0 || e.table >= CTRAJ_MAX_TABLES || !c->tables[e.table].n)
        return fail(CTRAJ_ESTATE, "honeycomb element %zu uses mesh table %d, which is not set", i, e.table);
      const HostTable& t = c->tables[e.table];
      int st = check_honeycomb(e, int(i), t.kind, t.n);
      if (st) return st;
    }
  }
  return CTRAJ_OK;
}

int enqueue_persistent(bool out, int mode, const Plan& P, const RunDev& R, int i, const Queue& Qin,
                       const Queue& Qnext, unsigned* order_buf, int sms, int interval, int service, cudaStream_t s,
                       int* launches, int lanes, int mpt, DoneRec* done) {
  const bool staged = P.lf[i].n_smem > 0;
  int kt = kPersistThreads, km = 1;
  const PersistKernel k = persist_kernel(out, P.lf[i].force, mode, staged, lanes, mpt, &kt, &km);
  const size_t smem =
      (staged ? size_t(P.lf[i].n_int) * sizeof(float4) : 0) + size_t(kt) * size_t(km) * sizeof(SwapSlot);
  CT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  unsigned* hist = order_buf;
  unsigned* order = hist + kOrderBuckets;
  CT_CUDA(cudaMemsetAsync(hist, 0, kOrderBuckets * sizeof(unsigned), s));
  k_order_count<<<sms, kOrderThreads, 0, s>>>(P, i, Qin, hist, P.lf[i].outward);
  k_order_scan<<<1, kOrderBuckets, 0, s>>>(hist);
  k_order_place<<<sms, kOrderThreads, 0, s>>>(P, i, Qin, hist, order, P.lf[i].outward);
  k<<<sms, kt, smem, s>>>(P, R, i, Qin, Qnext, lens_args(P, i, true), order, interval, service, done);
  CT_CUDA(cudaGetLastError());
  *launches += 4;
  if (done) {  // the molecules' ends, in full warps
    finish_kernel(mode)<<<sms * 8, kFinishThreads, 0, s>>>(P, R, i, Qin, Qnext, done, 0xFFFFFFFFu);
    CT_CUDA(cudaGetLastError());
    *launches += 1;
  }
  return CTRAJ_OK;
}


int validate_run(const ctraj_context* c, const ctraj_run_args* a) {
  if (!a) return fail(CTRAJ_EINVAL, "args is NULL");
  if (!c->have_beamline) return fail(CTRAJ_ESTATE, "ctraj_set_beamline was not called");
  if (a->n < 0 || a->n > int64_t(0x7fffffff)) return fail(CTRAJ_EINVAL, "n = %lld out of range [0, 2^31)", (long long)a->n);
  if (a->precision != 32 && a->precision != 64) return fail(CTRAJ_EINVAL, "precision must be 32 or 64");
  if (a->ic_mode == CTRAJ_IC_DEVICE_DRAW) {
    if (a->xdist.kind != CTRAJ_DIST_GAUSSIAN_POSITION && a->xdist.kind != CTRAJ_DIST_DISC_POSITION)
      return fail(CTRAJ_EINVAL, "unknown position distribution kind %d", a->xdist.kind);
    if (a->vdist.kind != CTRAJ_DIST_GAUSSIAN_VELOCITY)
      return fail(CTRAJ_EINVAL, "unknown velocity distribution kind %d", a->vdist.kind);
  } else if (a->ic_mode == CTRAJ_IC_HOST || a->ic_mode == CTRAJ_IC_DEVICE) {
    if (!a->ics && a->n > 0) return fail(CTRAJ_EINVAL, "ics is NULL");
  } else {
    return fail(CTRAJ_EINVAL, "unknown ic_mode %d", a->ic_mode);
  }
  if (a->out_mode < CTRAJ_OUT_NONE || a->out_mode > CTRAJ_OUT_DEVICE) return fail(CTRAJ_EINVAL, "bad out_mode");
  if (!a->counts) return fail(CTRAJ_EINVAL, "counts is NULL");
  return check_beamline(c);
}

// Shared by ctraj_run and ctraj_record: plan, ICs on the device, RunDev.
int prepare(ctraj_context* c, const ctraj_run_args* a, Plan& P, RunDev& R) {
  CT_CUDA(cudaSetDevice(c->device));
  int st;
  for (int k = 0; k < CTRAJ_MAX_TABLES; ++k) {
    HostTable& t = c->tables[k];
    if (t.n && !t.uploaded) {
      const size_t nb = align256(t.n * 8);
      const size_t cb = t.coef.empty() ? 0 : t.coef.size() * 8;
      const size_t vb = t.values.empty() ? 0 : t.values.size() * 8;
      if ((st = t.dev.ensure(nb + std::max(cb, vb)))) return st;
      CT_CUDA(cudaMemcpyAsync(t.dev.p, t.knots.data(), t.n * 8, cudaMemcpyHostToDevice, c->stream));
      if (cb) CT_CUDA(cudaMemcpyAsync(t.dev.as<char>(nb), t.coef.data(), cb, cudaMemcpyHostToDevice, c->stream));
      if (vb) CT_CUDA(cudaMemcpyAsync(t.dev.as<char>(nb), t.values.data(), vb, cudaMemcpyHostToDevice, c->stream));
      t.uploaded = true;
    }
  }
  if (c->lens_tables_dirty && (st = build_lens_tables(c))) return st;
  if ((st = build_plan(c, a, P))) return st;
  std::memset(&R, 0, sizeof R);
  R.n = a->n;
  R.rec_lens = -1;
  R.seed = a->seed;
  R.key = philox_key(a->seed);
  R.offset = a->offset;
  R.ic_mode = a->ic_mode;
  R.xd = a->xdist;
  R.vd = a->vdist;
  if (a->ic_mode == CTRAJ_IC_DEVICE_DRAW) {
    const double zd = a->xdist.kind == CTRAJ_DIST_DISC_POSITION ? a->xdist.p[1] : a->xdist.p[2];
    R.gap0f = P.n_el > 0 ? float(P.el[0].z0 - zd) : 0.f;
  } else if (a->ic_mode == CTRAJ_IC_HOST && a->n > 0) {
    const size_t b = size_t(a->n) * 6 * 8;
    if ((st = c->ics.ensure(b))) return st;
    CT_CUDA(cudaMemcpyAsync(c->ics.p, a->ics, b, cudaMemcpyHostToDevice, c->stream));
    R.ics = c->ics.as<double>();
  } else {
    R.ics = a->ics;
  }
  return CTRAJ_OK;
}

namespace {

// The persistent lens pass of a run on context c (its order buffer and tuning).
// count: the most entries Qin can hold (its count, or its capacity when the
// pass is enqueued without reading the count back); it sizes the entrant
// order and the molecules' end records.
int launch_persistent(ctraj_context* c, bool out, int mode, const Plan& P, const RunDev& R, int i, const Queue& Qin,
                      const Queue& Qnext, unsigned count, int* launches) {
  int st = c->lens_order.ensure((size_t(kOrderBuckets) + count) * sizeof(unsigned), 25);
  if (st) return st;
  // plain and batch passes without per-molecule outputs defer their molecules' ends
  DoneRec* done = nullptr;
  if (!out && (mode == kModePlain || mode == kModeBatch)) {
    if ((st = c->lens_done.ensure(size_t(count) * kDoneRecBytes, 25))) return st;
    done = c->lens_done.as<DoneRec>();
  }
  return enqueue_persistent(out, mode, P, R, i, Qin, Qnext, c->lens_order.as<unsigned>(), c->sm_count,
                            c->lens_interval, c->lens_service, c->stream, launches,
                            mode == kModeBatch ? c->batch_lens_threads : c->lens_threads, c->lens_molecules, done);
}

// k_front, then for each lens: read the lens queue's size and largest
// remaining step count (one small device-to-host copy), and launch
// ceil(max / chunk) chunk kernels that ping-pong between two queues while
// molecules leaving the lens collect in a third for the next lens.
// *left receives the molecules still in a lens afterwards (always 0).
template <bool k64, bool kOut, bool kRing = false>
int launch_all(ctraj_context* c, const Plan& P, const RunDev& R0, Queue* q, int* launches) {
  RunDev R = R0;  // ring recording fills in the staging buffers once the lens count is known
  c->run_max_steps = 0;
  unsigned ring_slots = 0;
  const int64_t n = R.n;
  cudaStream_t s = c->stream;
  if (c->timing) CT_CUDA(cudaEventRecord(c->ev[0], s));
  if (n > 0) {
    int st = launch_front(P, R, q[0], n, k64 ? 64 : 32, kOut, kRing ? kModeRing : kModePlain, c->front_threads,
                          c->sm_count, c->front_waves, s);
    if (st) return st;
    ++*launches;
  }
  if (c->timing) CT_CUDA(cudaEventRecord(c->ev[1], s));
  bool started = false;
  int cur = 0, alt = 1, nxt = 2;
  // The FP32 persistent pass needs nothing from the host mid-run: its
  // kernels read the lens queue's count on the device (and return at once
  // when it is 0), its buffers are sized for the queue's capacity, and the
  // largest step bound (a statistic) is copied back with the counts.  The
  // whole run is enqueued without a synchronisation.
  const bool async = !k64 && !kRing && c->lens_mode == CTRAJ_LENS_PERSISTENT;
  c->lens_async = async;
  for (int i = 0; i < P.n_el && n > 0; ++i) {
    if (P.el[i].type != CTRAJ_ELECTROSTATIC_LENS) continue;
    if (async) {
      if (c->timing && !started) CT_CUDA(cudaEventRecord(c->ev[2], s));
      started = true;
      CT_CUDA(cudaMemcpyAsync(c->host_lens + i, q[cur].max_steps, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
      CT_CUDA(cudaMemsetAsync(q[nxt].count, 0, kCtlWords * sizeof(unsigned), s));
      int st = launch_persistent(c, kOut, kModePlain, P, R, i, q[cur], q[nxt], unsigned(n), launches);
      if (st) return st;
      std::swap(cur, nxt);
      continue;
    }
    CT_CUDA(cudaMemcpyAsync(c->host_max, q[cur].count, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CT_CUDA(cudaStreamSynchronize(s));
    const unsigned count = c->host_max[0], max_steps = c->host_max[1];
    if (count == 0) break;  // no molecule reaches this lens, hence none reaches a later one
    c->run_max_steps = std::max(c->run_max_steps, max_steps);
    if (c->timing && !started) CT_CUDA(cudaEventRecord(c->ev[2], s));
    started = true;
    CT_CUDA(cudaMemsetAsync(q[nxt].count, 0, kCtlWords * sizeof(unsigned), s));
    const bool staged = !k64 && P.lf[i].n_smem > 0;
    const size_t smem = staged ? size_t(P.lf[i].n_int) * sizeof(float4) : 0;
    LensKernel kl = lens_kernel(k64, kOut, kRing, P.lf[i].force, staged);
    if (kRing && i == R.rec_lens) {
      // staging: per lens entrant (record slot) the records and five scalars
      R.rec_max = int(max_steps / unsigned(R.rec_stride)) + 3;
      const size_t recb = align256(size_t(count) * size_t(R.rec_max) * sizeof(float4));
      const size_t sb = align256(size_t(count) * 4);
      int st = c->rec_stage.ensure(recb + 5 * sb + 2 * align256(size_t(count) * 8), 25);
      if (st) return st;
      char* b = c->rec_stage.as<char>();
      R.rec = reinterpret_cast<float4*>(b);
      R.rec_n = reinterpret_cast<int32_t*>(b + recb);
      R.rec_last = reinterpret_cast<int32_t*>(b + recb + sb);
      R.rec_id = reinterpret_cast<int32_t*>(b + recb + 2 * sb);
      R.rec_t0 = reinterpret_cast<float*>(b + recb + 3 * sb);
      R.rec_vz = reinterpret_cast<float*>(b + recb + 4 * sb);
      R.rec_r0 = reinterpret_cast<unsigned long long*>(b + recb + 5 * sb);
      R.rec_m0 = reinterpret_cast<unsigned long long*>(b + recb + 5 * sb + align256(size_t(count) * 8));
      CT_CUDA(cudaMemsetAsync(R.rec_n, 0, sb, s));
      ring_slots = count;
    }
    if constexpr (!k64) {
      if (c->lens_mode == CTRAJ_LENS_PERSISTENT) {
        int st = launch_persistent(c, kOut, kRing ? kModeRing : kModePlain, P, R, i, q[cur], q[nxt], count, launches);
        if (st) return st;
        c->host_max[2 + i] = 0;  // no continuation queue
        std::swap(cur, nxt);
        continue;
      }
    }
    CT_CUDA(cudaFuncSetAttribute(kl, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
    const int64_t per_launch = int64_t(blocks_per_sm(kl, kLensThreads, smem)) * c->sm_count;
    const int grid =
        int(std::max<int64_t>(1, std::min<int64_t>(per_launch, (count + kLensThreads - 1) / kLensThreads)));
    // chunk lengths double from c->chunk up to c->chunk_max: molecules are
    // lost fastest right after the entrance, so compaction is frequent there
    // and launches are few in the long tail of survivors
    std::vector<int> lens_chunks;
    for (int64_t done = 0, len = c->chunk; done < int64_t(max_steps) || lens_chunks.empty();) {
      if (lens_chunks.size() == size_t(kMaxChunks))
        return fail(CTRAJ_ESTEPS, "lens element %d needs more than %d chunks", i, kMaxChunks);
      lens_chunks.push_back(int(len));
      done += len;
      len = std::min<int64_t>(std::max<int64_t>(len + 1, len * c->chunk_growth / 100), c->chunk_max);
    }
    const size_t nc = lens_chunks.size();
    CT_CUDA(cudaMemsetAsync(c->chunk_ctl.p, 0, nc * kCtlWords * sizeof(unsigned), s));
    const LensArgs la = lens_args(P, i, !k64);
    Queue in = q[cur];
    for (size_t k = 0; k < nc; ++k) {
      Queue out = q[alt];  // each chunk counts its output in its own slots: no reset in between
      out.count = c->chunk_ctl.as<unsigned>(k * kCtlWords * sizeof(unsigned));
      out.max_steps = out.count + 1;
      out.head = out.count + 2;
      kl<<<grid, kLensThreads, smem, s>>>(P, R, i, in, out, q[nxt], lens_chunks[k], la);
      CT_CUDA(cudaGetLastError());
      ++*launches;
      in = out;
      std::swap(cur, alt);
    }
    // the last chunk's continuation queue must be empty
    CT_CUDA(cudaMemcpyAsync(c->host_max + 2 + i, in.count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    std::swap(cur, nxt);  // the next lens starts from the molecules queued at its entrance
  }
  if (kRing && n > 0) {  // also when no molecule reached the lens: entrance losses
    int st = c->ring_part.ensure(2 * kRingBlocks * sizeof(unsigned long long));
    if (st) return st;
    unsigned long long* part = c->ring_part.as<unsigned long long>();
    k_ring_count<<<kRingBlocks, kRingThreads, 0, s>>>(R, ring_slots, part);
    k_ring_scan<<<1, kRingBlocks, 0, s>>>(R, part);
    k_ring_reserve<<<kRingBlocks, kRingThreads, 0, s>>>(R, ring_slots, part);
    CT_CUDA(cudaGetLastError());
    if constexpr (!k64) {
      k_ring_write<Mol32<false, false>><<<c->sm_count * 8, 256, 0, s>>>(P, R, ring_slots);
      CT_CUDA(cudaGetLastError());
      *launches += 1;
    }
    *launches += 3;
  }
  if (c->timing) {
    if (!started) CT_CUDA(cudaEventRecord(c->ev[2], s));
    CT_CUDA(cudaEventRecord(c->ev[3], s));
  }
  return CTRAJ_OK;
}

}  // namespace
}  // namespace ctraj

using namespace ctraj;

// ============================================================================
// C ABI
// ============================================================================
extern "C" {

int ctraj_version(void) { return CTRAJ_ABI_VERSION; }

const char* ctraj_last_error(void) { return g_error.c_str(); }

int ctraj_create(int device, ctraj_context** out) {
  if (!out) return fail(CTRAJ_EINVAL, "out is NULL");
  *out = nullptr;
  int n_dev = 0;
  CT_CUDA(cudaGetDeviceCount(&n_dev));
  if (device < 0 || device >= n_dev) return fail(CTRAJ_EINVAL, "device %d not present (%d devices)", device, n_dev);
  CT_CUDA(cudaSetDevice(device));
  auto* c = new ctraj_context();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
  for (int k = 0; k < 4 && e == cudaSuccess; ++k) e = cudaEventCreate(&c->ev[k]);
  if (e == cudaSuccess) e = cudaMallocHost(&c->host_max, (2 + CTRAJ_MAX_ELEMENTS) * sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMallocHost(&c->host_lens, CTRAJ_MAX_ELEMENTS * sizeof(unsigned));
  c->stream = c->own_stream;
  if (e != cudaSuccess) {
    ctraj_destroy(c);
    return fail(CTRAJ_ECUDA, "context setup: %s", cudaGetErrorString(e));
  }
  int st = c->qctl.ensure(4096);
  if (!st) st = c->chunk_ctl.ensure(size_t(kMaxChunks) * kCtlWords * sizeof(unsigned));
  if (st) {
    std::string msg = g_error;
    ctraj_destroy(c);  // releases whatever was set up
    g_error = msg;
    return st;
  }
  *out = c;
  return CTRAJ_OK;
}

int ctraj_destroy(ctraj_context* c) {
  if (!c) return CTRAJ_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  for (auto& t : c->tables) t.dev.release();
  c->lens_tables.release();
  for (auto& q : c->queue) q.release();
  c->qctl.release();
  c->ics.release();
  c->outs.release();
  c->rec_rows.release();
  c->rec_ids.release();
  c->rec_count.release();
  c->chunk_ctl.release();
  c->rec_stage.release();
  c->ring_ent.release();
  c->lens_order.release();
  c->lens_done.release();
  c->sweep_done.release();
  c->ring_part.release();
  c->sweep_order.release();
  if (c->sweep_exec) cudaGraphExecDestroy(c->sweep_exec);
  for (int t = 0; t < CTRAJ_MAX_TABLES; ++t) {
    if (c->side[t]) cudaStreamSynchronize(c->side[t]);
    if (c->side[t]) cudaStreamDestroy(c->side[t]);
    if (c->join[t]) cudaEventDestroy(c->join[t]);
  }
  if (c->fork) cudaEventDestroy(c->fork);
  c->sweep_tables.release();
  c->sweep_cfg.release();
  c->sweep_ctl.release();
  for (auto& q : c->sweep_queue) q.release();
  if (c->sweep_host) cudaFreeHost(c->sweep_host);
  c->soft_table.release();
  c->soft_queue.release();
  c->soft_ckpt.release();
  c->soft_ctl.release();
  c->soft_contrib.release();
  c->soft_seg.release();
  c->soft_post.release();
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  if (c->peer) ctraj_destroy(c->peer);
  cudaSetDevice(c->device);
  c->l2_flush.release();
  c->group_ctl.release();
  c->group_ics.release();
  if (c->group_host) cudaFreeHost(c->group_host);
  if (c->batch_ev) cudaEventDestroy(c->batch_ev);
  if (c->host_max) cudaFreeHost(c->host_max);
  if (c->host_lens) cudaFreeHost(c->host_lens);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
  return CTRAJ_OK;
}

int ctraj_set_tuning(ctraj_context* c, const ctraj_tuning* t) {
  if (!c || !t) return fail(CTRAJ_EINVAL, "NULL argument");
  if (t->chunk_first < 1 || t->chunk_max < t->chunk_first || t->chunk_max > 1000000 ||
      t->chunk_growth < 100 || t->chunk_growth > 1000 || t->front_waves < 1 || t->front_waves > 64 ||
      (t->lens_mode != CTRAJ_LENS_PERSISTENT && t->lens_mode != CTRAJ_LENS_CHUNKED) || t->lens_interval < 1 ||
      t->lens_interval > 100000 || (t->front_threads != 128 && t->front_threads != 256 && t->front_threads != 512) ||
      t->batch_group < 1 || t->batch_group > CTRAJ_MAX_BATCH_GROUP ||
      (t->lens_threads != 512 && t->lens_threads != 768 && t->lens_threads != 1024) ||
      (t->lens_molecules != 1 && t->lens_molecules != 2) ||
      (t->batch_lens_threads != 512 && t->batch_lens_threads != 768 && t->batch_lens_threads != 1024) ||
      t->lens_service < 1 || t->lens_service > 100000)
    return fail(CTRAJ_EINVAL,
                "tuning out of range (chunk_first %d, chunk_growth %d, chunk_max %d, front_waves %d, lens_mode %d, "
                "lens_interval %d, front_threads %d, batch_group %d, lens_threads %d, lens_molecules %d, "
                "batch_lens_threads %d, lens_service %d)",
                t->chunk_first, t->chunk_growth, t->chunk_max, t->front_waves, t->lens_mode, t->lens_interval,
                t->front_threads, t->batch_group, t->lens_threads, t->lens_molecules, t->batch_lens_threads,
                t->lens_service);
  c->chunk = t->chunk_first;
  c->chunk_growth = t->chunk_growth;
  c->chunk_max = t->chunk_max;
  c->front_waves = t->front_waves;
  c->lens_mode = t->lens_mode;
  c->lens_interval = t->lens_interval;
  c->front_threads = t->front_threads;
  c->batch_group = t->batch_group;
  c->lens_threads = t->lens_threads;
  c->lens_molecules = t->lens_molecules;
  c->batch_lens_threads = t->batch_lens_threads;
  c->lens_service = t->lens_service;
  ++c->generation;
  return CTRAJ_OK;
}

int ctraj_get_tuning(ctraj_context* c, ctraj_tuning* t) {
  if (!c || !t) return fail(CTRAJ_EINVAL, "NULL argument");
  t->chunk_first = c->chunk;
  t->chunk_growth = c->chunk_growth;
  t->chunk_max = c->chunk_max;
  t->front_waves = c->front_waves;
  t->lens_mode = c->lens_mode;
  t->lens_interval = c->lens_interval;
  t->front_threads = c->front_threads;
  t->batch_group = c->batch_group;
  t->lens_threads = c->lens_threads;
  t->lens_molecules = c->lens_molecules;
  t->batch_lens_threads = c->batch_lens_threads;
  t->lens_service = c->lens_service;
  return CTRAJ_OK;
}

int ctraj_set_stream(ctraj_context* c, void* stream) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  c->stream = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
  ++c->generation;
  return CTRAJ_OK;
}

int ctraj_synchronize(ctraj_context* c) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  CT_CUDA(cudaSetDevice(c->device));
  CT_CUDA(cudaStreamSynchronize(c->stream));
  return CTRAJ_OK;
}

int ctraj_set_beamline(ctraj_context* c, const ctraj_element* el, int32_t n_el, int32_t n_labels) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  if (n_el < 0 || n_el > CTRAJ_MAX_ELEMENTS) return fail(CTRAJ_EINVAL, "n_elements %d out of range", n_el);
  if (n_labels < 0 || n_labels > CTRAJ_MAX_LABELS) return fail(CTRAJ_EINVAL, "n_labels %d out of range", n_labels);
  if (n_el > 0 && !el) return fail(CTRAJ_EINVAL, "elements is NULL");
  for (int i = 0; i < n_el; ++i) {
    const ctraj_element& e = el[i];
    if (e.type < CTRAJ_CIRCULAR_APERTURE || e.type > CTRAJ_HONEYCOMB)
      return fail(CTRAJ_EINVAL, "element %d: unknown type %d", i, e.type);
    if (e.label < -1 || e.label >= n_labels || e.label_inside < -1 || e.label_inside >= n_labels)
      return fail(CTRAJ_EINVAL, "element %d: label out of range", i);
    if (i > 0 && e.z0 < el[i - 1].z0) return fail(CTRAJ_EINVAL, "elements are not sorted by z0 (element %d)", i);
    if ((e.type == CTRAJ_ELECTROSTATIC_LENS || e.type == CTRAJ_HONEYCOMB) && (e.table < 0 || e.table >= CTRAJ_MAX_TABLES))
      return fail(CTRAJ_EINVAL, "element %d: table id %d out of range", i, e.table);
  }
  // the beamline already set (a caller that sets it before every run): its
  // device tables and everything derived from it stay valid
  if (c->have_beamline && c->n_labels == n_labels && c->elements.size() == size_t(n_el) &&
      (n_el == 0 || std::memcmp(c->elements.data(), el, size_t(n_el) * sizeof(ctraj_element)) == 0))
    return CTRAJ_OK;
  c->elements.assign(el, el + n_el);
  c->n_labels = n_labels;
  c->have_beamline = true;
  c->lens_tables_dirty = true;
  ++c->generation;
  return CTRAJ_OK;
}

// The table already set under this id, bit for bit (knots and coefficients
// or values).
static bool same_table(const HostTable& ht, const ctraj_force_table* t) {
  if (ht.n == 0 || ht.kind != t->kind || ht.n != t->n_knots || !t->knots) return false;
  if (std::memcmp(ht.knots.data(), t->knots, size_t(t->n_knots) * sizeof(double)) != 0) return false;
  if (t->kind == CTRAJ_TABLE_STARK_SPLINE)
    return t->coef && ht.coef.size() == size_t(t->n_knots - 1) * 4 &&
           std::memcmp(ht.coef.data(), t->coef, ht.coef.size() * sizeof(double)) == 0;
  return t->values && ht.values.size() == size_t(t->n_knots) &&
         std::memcmp(ht.values.data(), t->values, ht.values.size() * sizeof(double)) == 0;
}

int ctraj_set_force_table(ctraj_context* c, int32_t id, const ctraj_force_table* t) {
  if (!c || !t) return fail(CTRAJ_EINVAL, "NULL argument");
  if (id < 0 || id >= CTRAJ_MAX_TABLES) return fail(CTRAJ_EINVAL, "table id %d out of range", id);
  // the table already set (validated then): nothing to copy, rebuild or upload
  if (same_table(c->tables[id], t)) return CTRAJ_OK;
  if (t->kind == CTRAJ_TABLE_MESH) {
    if (t->n_knots < 1 || !t->knots || !t->values) return fail(CTRAJ_EINVAL, "mesh table needs at least one cell");
    for (int j = 0; j < t->n_knots; ++j)
      if (!std::isfinite(t->knots[j]) || !std::isfinite(t->values[j]))
        return fail(CTRAJ_EINVAL, "mesh table: cell %d is not finite", j);
  } else {
    if (t->n_knots < 2 || !t->knots) return fail(CTRAJ_EINVAL, "table needs at least 2 knots");
    if (t->kind == CTRAJ_TABLE_STARK_SPLINE && !t->coef) return fail(CTRAJ_EINVAL, "spline table without coef");
    if (t->kind == CTRAJ_TABLE_RADIAL_LINEAR && !t->values) return fail(CTRAJ_EINVAL, "radial table without values");
    if (t->kind != CTRAJ_TABLE_STARK_SPLINE && t->kind != CTRAJ_TABLE_RADIAL_LINEAR)
      return fail(CTRAJ_EINVAL, "unknown table kind %d", t->kind);
    const double h = (t->knots[t->n_knots - 1] - t->knots[0]) / double(t->n_knots - 1);
    if (!(h > 0)) return fail(CTRAJ_EINVAL, "table knots must ascend");
    for (int j = 1; j < t->n_knots; ++j)
      if (std::fabs((t->knots[j] - t->knots[j - 1]) - h) > 1e-6 * h)
        return fail(CTRAJ_EINVAL, "table knots must be uniformly spaced (knot %d)", j);
  }
  HostTable& ht = c->tables[id];
  ht.kind = t->kind;
  ht.n = t->n_knots;
  ht.knots.assign(t->knots, t->knots + t->n_knots);
  ht.coef.clear();
  ht.values.clear();
  if (t->kind == CTRAJ_TABLE_STARK_SPLINE) ht.coef.assign(t->coef, t->coef + size_t(t->n_knots - 1) * 4);
  else ht.values.assign(t->values, t->values + t->n_knots);
  ht.uploaded = false;
  c->lens_tables_dirty = true;
  ++c->generation;
  return CTRAJ_OK;
}

// ctraj_run, and with ring != NULL ctraj_run_ring.
static int run_impl(ctraj_context* c, const ctraj_run_args* a, ctraj_run_stats* stats, const ctraj_ring* ring) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  int st = validate_run(c, a);
  if (st) return st;
  Plan P;
  RunDev R;
  if ((st = prepare(c, a, P, R))) return st;
  if (ring) {
    if (a->precision != 32) return fail(CTRAJ_EINVAL, "ring recording runs in precision 32 only");
    if (!ring->rows || !ring->index || !ring->heads || ring->capacity_rows < 1 || ring->capacity_molecules < 1 ||
        ring->stride < 1)
      return fail(CTRAJ_EINVAL, "bad ring (buffers, capacities >= 1, stride >= 1)");
    if (ring->lens != P.first_lens || P.first_lens >= P.n_el)
      return fail(CTRAJ_EINVAL, "the recorded lens must be the first lens of the beamline (element %d)",
                  P.first_lens);
    R.rec_lens = ring->lens;
    R.rec_stride = ring->stride;
    R.rec_entrance_label = P.el[ring->lens].label;
    R.ring = *ring;
    // list of the molecules stopped by the entrance test: count | ids | rows taken | entries taken
    const size_t m = size_t(std::max<int64_t>(a->n, 1));
    if ((st = c->ring_ent.ensure(256 + align256(m * 4) + 2 * align256(m * 8)))) return st;
    char* b = c->ring_ent.as<char>();
    R.ent_count = reinterpret_cast<unsigned*>(b);
    R.ent_id = reinterpret_cast<int32_t*>(b + 256);
    R.ent_r0 = reinterpret_cast<unsigned long long*>(b + 256 + align256(m * 4));
    R.ent_m0 = reinterpret_cast<unsigned long long*>(b + 256 + align256(m * 4) + align256(m * 8));
    CT_CUDA(cudaMemsetAsync(R.ent_count, 0, 4, c->stream));
  }
  const int64_t n = a->n;
  const size_t cap = size_t(std::max<int64_t>(n, 1));
  int n_lens = 0;
  for (int i = 0; i < P.n_el; ++i) n_lens += P.el[i].type == CTRAJ_ELECTROSTATIC_LENS;
  // two queues per lens (chunk ping-pong) plus one collecting the next lens's entrants
  const int n_queues = n_lens == 0 ? 1 : (n_lens == 1 ? 2 : 3);
  for (int k = 0; k < n_queues; ++k)
    if ((st = c->queue[k].ensure(queue_bytes(cap, a->precision, ring != nullptr)))) return st;
  unsigned* ctl = c->qctl.as<unsigned>();
  unsigned long long* counts = c->qctl.as<unsigned long long>(256);
  unsigned long long* dstats = c->qctl.as<unsigned long long>(256 + 8 * (CTRAJ_MAX_LABELS + 1));
  // without a third buffer the next-lens queue aliases queue 1's storage: it is
  // never written, because nothing follows the last lens
  Queue q[3];
  for (int k = 0; k < 3; ++k)
    layout_queue(&c->queue[std::min(k, n_queues - 1)], cap, a->precision, ctl + kCtlWords * k, &q[k],
                 ring != nullptr);
  CT_CUDA(cudaMemsetAsync(c->qctl.p, 0, 4096, c->stream));
  R.counts = counts;
  R.stats = dstats;
  const bool out = a->out_mode != CTRAJ_OUT_NONE;
  if (a->out_mode == CTRAJ_OUT_HOST && n > 0) {
    const size_t b = align256(n * 4) * 2 + align256(n * 8) + align256(n * 80);
    if ((st = c->outs.ensure(b))) return st;
    R.out_label = a->out_label ? c->outs.as<int32_t>(0) : nullptr;
    R.out_rows = a->out_rows ? c->outs.as<int32_t>(align256(n * 4)) : nullptr;
    R.out_margin = a->out_margin ? c->outs.as<double>(2 * align256(n * 4)) : nullptr;
    R.out_final = a->out_final ? c->outs.as<double>(2 * align256(n * 4) + align256(n * 8)) : nullptr;
  } else if (a->out_mode == CTRAJ_OUT_DEVICE) {
    R.out_label = a->out_label;
    R.out_rows = a->out_rows;
    R.out_margin = a->out_margin;
    R.out_final = a->out_final;
  }
  int launches = 0;
  std::memset(c->host_max, 0, (2 + CTRAJ_MAX_ELEMENTS) * sizeof(unsigned));
  std::memset(c->host_lens, 0, CTRAJ_MAX_ELEMENTS * sizeof(unsigned));
  c->lens_async = false;
  c->timing = a->timing != 0;
  if (ring)
    st = out ? launch_all<false, true, true>(c, P, R, q, &launches)
             : launch_all<false, false, true>(c, P, R, q, &launches);
  else if (a->precision == 32)
    st = out ? launch_all<false, true>(c, P, R, q, &launches) : launch_all<false, false>(c, P, R, q, &launches);
  else
    st = out ? launch_all<true, true>(c, P, R, q, &launches) : launch_all<true, false>(c, P, R, q, &launches);
  if (st) return st;
  unsigned long long hc[CTRAJ_MAX_LABELS + 1], hs[kStatCount];
  CT_CUDA(cudaMemcpyAsync(hc, counts, sizeof hc, cudaMemcpyDeviceToHost, c->stream));
  CT_CUDA(cudaMemcpyAsync(hs, dstats, sizeof hs, cudaMemcpyDeviceToHost, c->stream));
  if (a->out_mode == CTRAJ_OUT_HOST && n > 0) {
    if (a->out_label) CT_CUDA(cudaMemcpyAsync(a->out_label, R.out_label, n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (a->out_rows) CT_CUDA(cudaMemcpyAsync(a->out_rows, R.out_rows, n * 4, cudaMemcpyDeviceToHost, c->stream));
    if (a->out_margin) CT_CUDA(cudaMemcpyAsync(a->out_margin, R.out_margin, n * 8, cudaMemcpyDeviceToHost, c->stream));
    if (a->out_final) CT_CUDA(cudaMemcpyAsync(a->out_final, R.out_final, n * 80, cudaMemcpyDeviceToHost, c->stream));
  }
  CT_CUDA(cudaStreamSynchronize(c->stream));
  if (c->lens_async)
    for (int i = 0; i < P.n_el; ++i) c->run_max_steps = std::max(c->run_max_steps, c->host_lens[i]);
  for (int i = 0; i < P.n_el; ++i)
    if (c->host_max[2 + i] != 0)
      return fail(CTRAJ_ECUDA, "internal error: %u molecules left inside lens element %d",
                  c->host_max[2 + i], i);
  for (int k = 0; k <= c->n_labels; ++k) a->counts[k] = int64_t(hc[k]);
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->molecules = n;
    stats->molecule_steps = int64_t(hs[kStatSteps]);
    stats->lens_steps = int64_t(hs[kStatLensSteps]);
    stats->max_lens_steps = int32_t(c->run_max_steps);
    if (a->precision == 32)
      for (int i = 0; i < P.n_el; ++i)
        stats->linear_tables += P.el[i].type == CTRAJ_ELECTROSTATIC_LENS && P.lf[i].force == kForceStark2Lin;
    stats->edge_band = (a->precision == 64 || out) ? int64_t(hs[kStatEdgeBand]) : -1;
    stats->table_range = int64_t(hs[kStatTableRange]);
    stats->bad_steps = int64_t(hs[kStatBadSteps]);
    stats->kernels = launches;
    if (c->timing) {
      stats->timed = 1;
      CT_CUDA(cudaEventElapsedTime(&stats->front_ms, c->ev[0], c->ev[1]));
      CT_CUDA(cudaEventElapsedTime(&stats->lens_ms, c->ev[2], c->ev[3]));
    }
  }
  if (hs[kStatRangeError])
    return fail(CTRAJ_ERANGE, "%llu molecules looked up the lens table above its last knot "
                "(interp1d would raise ValueError)", hs[kStatRangeError]);
  if (hs[kStatBadSteps])
    return fail(CTRAJ_ESTEPS, "%llu molecules have a non-finite or oversize lens step count rint(L/dz)",
                hs[kStatBadSteps]);
  return CTRAJ_OK;
}

int ctraj_run(ctraj_context* c, const ctraj_run_args* a, ctraj_run_stats* stats) {
  return run_impl(c, a, stats, nullptr);
}

// ---------------------------------------------------------------------------
// Grouped batches: consecutive runs of ctraj_run_batch whose molecules share
// one persistent lens pass per lens.  A lens pass ends with a long tail in
// which only the slowest molecules (the most RK4 steps) are left; sharing the
// pass lets that tail overlap the bulk of the other runs, so the group costs
// one tail instead of one per run.  Each molecule carries its run's index in
// the group; every count and stat goes to its run's own slots, so each run's
// results are those of ctraj_run.
// ---------------------------------------------------------------------------

// Whether run a can share the lens pass of a group whose first run is first.
static bool group_member(const ctraj_context* c, const ctraj_run_args* a, const ctraj_run_args* first) {
  return a->precision == 32 && a->out_mode == CTRAJ_OUT_NONE && c->lens_mode == CTRAJ_LENS_PERSISTENT &&
         a->g == first->g;
}

// Runs a[0..g) as one group on context c; per-run counts go to a[j].counts
// and stats to stats[j] (may be NULL).  flush > 0: that many bytes of the
// context's scratch are written before each run's front.  Returns the status
// of the first failing run (by index) and its index in *failed (-1 if none).
static int run_group(ctraj_context* c, const ctraj_run_args* a, int g, ctraj_run_stats* stats, uint64_t flush,
                     int* failed) {
  *failed = 0;
  int st;
  for (int j = 0; j < g; ++j) {
    *failed = j;
    if ((st = validate_run(c, &a[j]))) return st;
  }
  *failed = 0;
  CT_CUDA(cudaSetDevice(c->device));
  cudaStream_t s = c->stream;
  int64_t total = 0;
  size_t ic_bytes = 0;
  for (int j = 0; j < g; ++j) {
    total += a[j].n;
    if (a[j].ic_mode == CTRAJ_IC_HOST && a[j].n > 0) ic_bytes += align256(size_t(a[j].n) * 6 * 8);
  }
  if (total > int64_t(0x7fffffff)) return fail(CTRAJ_EINVAL, "a batch group holds more than 2^31 molecules");
  // per-run counts (n_labels + 1 words each, the stride tally_cfg uses) then
  // per-run stats (kStatCount each)
  const size_t cw = size_t(c->n_labels + 1), words = size_t(g) * (cw + kStatCount);
  if ((st = c->group_ctl.ensure(words * 8))) return st;
  if (words > c->group_host_words) {
    if (c->group_host) cudaFreeHost(c->group_host);
    c->group_host = nullptr;
    c->group_host_words = 0;
    CT_CUDA(cudaMallocHost(&c->group_host, words * 8));
    c->group_host_words = words;
  }
  if (ic_bytes && (st = c->group_ics.ensure(ic_bytes, 25))) return st;
  unsigned long long* run_counts = c->group_ctl.as<unsigned long long>();
  unsigned long long* run_stats = run_counts + size_t(g) * cw;
  // per run: plan and RunDev (host initial conditions go to their own slice)
  Plan P;
  std::vector<RunDev> R(g);
  size_t ic_off = 0;
  for (int j = 0; j < g; ++j) {
    ctraj_run_args aj = a[j];
    if (aj.ic_mode == CTRAJ_IC_HOST && aj.n > 0) {
      double* dst = c->group_ics.as<double>(ic_off);
      CT_CUDA(cudaMemcpyAsync(dst, aj.ics, size_t(aj.n) * 6 * 8, cudaMemcpyHostToDevice, s));
      ic_off += align256(size_t(aj.n) * 6 * 8);
      aj.ic_mode = CTRAJ_IC_DEVICE;
      aj.ics = dst;
    }
    if ((st = prepare(c, &aj, P, R[j]))) return st;
    R[j].counts = run_counts + size_t(j) * cw;
    R[j].stats = run_stats + size_t(j) * kStatCount;
    R[j].run_tag = j;
  }
  // one set of lens queues for the group, entries tagged with their run
  const size_t cap = size_t(std::max<int64_t>(total, 1));
  int n_lens = 0;
  for (int i = 0; i < P.n_el; ++i) n_lens += P.el[i].type == CTRAJ_ELECTROSTATIC_LENS;
  const int n_queues = n_lens == 0 ? 1 : (n_lens == 1 ? 2 : 3);
  for (int k = 0; k < n_queues; ++k)
    if ((st = c->queue[k].ensure(queue_bytes(cap, 32, true)))) return st;
  unsigned* ctl = c->qctl.as<unsigned>();
  Queue q[3];
  for (int k = 0; k < 3; ++k)
    layout_queue(&c->queue[std::min(k, n_queues - 1)], cap, 32, ctl + kCtlWords * k, &q[k], true);
  CT_CUDA(cudaMemsetAsync(c->qctl.p, 0, 4096, s));
  CT_CUDA(cudaMemsetAsync(run_counts, 0, words * 8, s));
  bool timing = false;
  for (int j = 0; j < g; ++j) timing = timing || a[j].timing;
  int launches = 0;
  c->timing = timing;
  if (timing) CT_CUDA(cudaEventRecord(c->ev[0], s));
  for (int j = 0; j < g; ++j) {
    if (flush) CT_CUDA(cudaMemsetAsync(c->l2_flush.p, j & 0xff, size_t(flush), s));
    if (a[j].n == 0) continue;
    if ((st = launch_front(P, R[j], q[0], a[j].n, 32, false, kModeBatch, c->front_threads, c->sm_count,
                           c->front_waves, s)))
      return st;
    ++launches;
  }
  const int fronts = launches;
  if (timing) CT_CUDA(cudaEventRecord(c->ev[1], s));
  RunDev Rg = R[0];  // the lens passes: tallies and stats per run
  Rg.cfg_counts = run_counts;
  Rg.cfg_stats = run_stats;
  Rg.counts = nullptr;
  Rg.stats = nullptr;
  bool started = false;
  int cur = 0, nxt = 2;
  // enqueued without a synchronisation, as a single run's persistent pass
  // (launch_all): the kernels read the queue counts on the device
  for (int i = 0; i < P.n_el && total > 0; ++i) {
    if (P.el[i].type != CTRAJ_ELECTROSTATIC_LENS) continue;
    if (timing && !started) CT_CUDA(cudaEventRecord(c->ev[2], s));
    started = true;
    CT_CUDA(cudaMemsetAsync(q[nxt].count, 0, kCtlWords * sizeof(unsigned), s));
    if ((st = launch_persistent(c, false, kModeBatch, P, Rg, i, q[cur], q[nxt], unsigned(total), &launches)))
      return st;
    std::swap(cur, nxt);
  }
  if (timing) {
    if (!started) CT_CUDA(cudaEventRecord(c->ev[2], s));
    CT_CUDA(cudaEventRecord(c->ev[3], s));
  }
  CT_CUDA(cudaMemcpyAsync(c->group_host, run_counts, words * 8, cudaMemcpyDeviceToHost, s));
  CT_CUDA(cudaStreamSynchronize(s));
  float front_ms = 0.f, lens_ms = 0.f;
  if (timing) {
    CT_CUDA(cudaEventElapsedTime(&front_ms, c->ev[0], c->ev[1]));
    CT_CUDA(cudaEventElapsedTime(&lens_ms, c->ev[2], c->ev[3]));
  }
  int linear = 0;
  for (int i = 0; i < P.n_el; ++i) linear += P.el[i].type == CTRAJ_ELECTROSTATIC_LENS && P.lf[i].force == kForceStark2Lin;
  int status = CTRAJ_OK;
  *failed = -1;
  for (int j = 0; j < g; ++j) {
    const unsigned long long* hc = c->group_host + size_t(j) * cw;
    const unsigned long long* hs = c->group_host + size_t(g) * cw + size_t(j) * kStatCount;
    for (int k = 0; k <= c->n_labels; ++k) a[j].counts[k] = int64_t(hc[k]);
    if (stats) {
      ctraj_run_stats& o = stats[j];
      std::memset(&o, 0, sizeof o);
      o.molecules = a[j].n;
      o.molecule_steps = int64_t(hs[kStatSteps]);
      o.lens_steps = int64_t(hs[kStatLensSteps]);
      o.max_lens_steps = int32_t(hs[kStatMaxSteps]);
      o.linear_tables = linear;
      o.edge_band = -1;
      o.table_range = int64_t(hs[kStatTableRange]);
      o.bad_steps = int64_t(hs[kStatBadSteps]);
      // each run its front launch; the group's shared launches are credited to its first run
      o.kernels = (a[j].n > 0 ? 1 : 0) + (j == 0 ? launches - fronts : 0);
      if (timing) {  // the group's kernel times, shared out evenly
        o.timed = 1;
        o.front_ms = front_ms / float(g);
        o.lens_ms = lens_ms / float(g);
      }
    }
    if (status == CTRAJ_OK && hs[kStatRangeError]) {
      status = fail(CTRAJ_ERANGE, "%llu molecules looked up the lens table above its last knot "
                    "(interp1d would raise ValueError)", hs[kStatRangeError]);
      *failed = j;
    } else if (status == CTRAJ_OK && hs[kStatBadSteps]) {
      status = fail(CTRAJ_ESTEPS, "%llu molecules have a non-finite or oversize lens step count rint(L/dz)",
                    hs[kStatBadSteps]);
      *failed = j;
    }
  }
  return status;
}

// One lane of a pipelined batch: groups lane, lane + 2, ... of `groups`
// (first run, run count) on context x.
struct BatchLane {
  int status = CTRAJ_OK;
  int run = -1;
  std::string error;
};

static void batch_lane(ctraj_context* x, const ctraj_run_args* a, const std::vector<std::pair<int, int>>* groups,
                       int lane, ctraj_run_stats* stats, uint64_t flush, BatchLane* out) {
  int st = CTRAJ_OK;
  int run = -1;
  if (cudaSetDevice(x->device) != cudaSuccess) st = fail(CTRAJ_ECUDA, "cudaSetDevice(%d) failed", x->device);
  if (!st && flush) st = x->l2_flush.ensure(size_t(flush));
  for (size_t gi = size_t(lane); !st && gi < groups->size(); gi += 2) {
    const int k = (*groups)[gi].first, g = (*groups)[gi].second;
    run = k;
    if (g > 1) {
      int bad = -1;
      st = run_group(x, a + k, g, stats ? stats + k : nullptr, flush, &bad);
      if (st) run = k + std::max(bad, 0);
      continue;
    }
    if (flush) {
      const cudaError_t e = cudaMemsetAsync(x->l2_flush.p, k & 0xff, size_t(flush), x->stream);
      if (e != cudaSuccess) st = fail(CTRAJ_ECUDA, "L2 flush: %s", cudaGetErrorString(e));
    }
    if (!st) st = run_impl(x, a + k, stats ? stats + k : nullptr, nullptr);
  }
  if (st) {
    out->status = st;
    out->run = run;
    out->error = g_error;
  }
}

// The second lane's context: same device, and the beamline, tables and
// tuning of c (copied again whenever c's generation moved).
static int batch_peer(ctraj_context* c) {
  if (!c->peer) {
    int st = ctraj_create(c->device, &c->peer);
    if (st) return st;
    c->peer_generation = ~uint64_t(0);
  }
  ctraj_context* p = c->peer;
  if (c->peer_generation != c->generation) {
    p->elements = c->elements;
    p->n_labels = c->n_labels;
    p->have_beamline = c->have_beamline;
    for (int t = 0; t < CTRAJ_MAX_TABLES; ++t) {
      p->tables[t].kind = c->tables[t].kind;
      p->tables[t].n = c->tables[t].n;
      p->tables[t].knots = c->tables[t].knots;
      p->tables[t].coef = c->tables[t].coef;
      p->tables[t].values = c->tables[t].values;
      p->tables[t].uploaded = false;
    }
    p->lens_tables_dirty = true;
    p->chunk = c->chunk;
    p->chunk_growth = c->chunk_growth;
    p->chunk_max = c->chunk_max;
    p->front_waves = c->front_waves;
    p->lens_mode = c->lens_mode;
    p->lens_interval = c->lens_interval;
    p->front_threads = c->front_threads;
    p->batch_group = c->batch_group;
    p->lens_threads = c->lens_threads;
    p->lens_molecules = c->lens_molecules;
    p->batch_lens_threads = c->batch_lens_threads;
    p->lens_service = c->lens_service;
    ++p->generation;
    c->peer_generation = c->generation;
  }
  return CTRAJ_OK;
}

int ctraj_run_batch(ctraj_context* c, const ctraj_run_args* a, int32_t n_runs, ctraj_run_stats* stats,
                    uint64_t l2_flush_bytes) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  if (n_runs < 0 || (n_runs > 0 && !a)) return fail(CTRAJ_EINVAL, "bad batch (n_runs %d)", n_runs);
  if (l2_flush_bytes > (uint64_t(1) << 34)) return fail(CTRAJ_EINVAL, "l2_flush_bytes above 16 GiB");
  if (n_runs == 0) return CTRAJ_OK;
  CT_CUDA(cudaSetDevice(c->device));
  // consecutive runs form groups of up to batch_group that share lens passes
  std::vector<std::pair<int, int>> groups;
  for (int k = 0; k < n_runs;) {
    int g = 1;
    if (c->batch_group > 1 && a[k].n >= 0 && group_member(c, &a[k], &a[k])) {
      int64_t total = a[k].n;
      while (g < c->batch_group && k + g < n_runs && a[k + g].n >= 0 && group_member(c, &a[k + g], &a[k]) &&
             total + a[k + g].n <= int64_t(0x7fffffff)) {
        total += a[k + g].n;
        ++g;
      }
    }
    groups.emplace_back(k, g);
    k += g;
  }
  BatchLane lanes[2];
  if (groups.size() == 1) {
    batch_lane(c, a, &groups, 0, stats, l2_flush_bytes, &lanes[0]);
  } else {
    int st = batch_peer(c);
    if (st) return st;
    if (!c->batch_ev) CT_CUDA(cudaEventCreateWithFlags(&c->batch_ev, cudaEventDisableTiming));
    if (!c->peer->batch_ev) CT_CUDA(cudaEventCreateWithFlags(&c->peer->batch_ev, cudaEventDisableTiming));
    // the batch starts after the work already queued on ctx's stream
    CT_CUDA(cudaEventRecord(c->batch_ev, c->stream));
    CT_CUDA(cudaStreamWaitEvent(c->peer->stream, c->batch_ev, 0));
    bool threaded = true;
    std::thread second;
    try {
      second = std::thread(batch_lane, c->peer, a, &groups, 1, stats, l2_flush_bytes, &lanes[1]);
    } catch (const std::system_error&) {
      threaded = false;  // no thread to be had: the lanes run one after the other
    }
    batch_lane(c, a, &groups, 0, stats, l2_flush_bytes, &lanes[0]);
    if (threaded) second.join();
    else batch_lane(c->peer, a, &groups, 1, stats, l2_flush_bytes, &lanes[1]);
    // and later work on ctx's stream after all of it
    CT_CUDA(cudaEventRecord(c->peer->batch_ev, c->peer->stream));
    CT_CUDA(cudaStreamWaitEvent(c->stream, c->peer->batch_ev, 0));
  }
  const BatchLane* bad = nullptr;
  for (const BatchLane& l : lanes)
    if (l.status && (!bad || l.run < bad->run)) bad = &l;
  if (bad) return fail(bad->status, "batch run %d: %s", bad->run, bad->error.c_str());
  return CTRAJ_OK;
}

int ctraj_plane(ctraj_context* c, const ctraj_run_args* a, const int64_t* ids, int64_t n_ids, double z_plane,
                double* out) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  int st = validate_run(c, a);
  if (st) return st;
  if (n_ids < 0 || (n_ids > 0 && (!ids || !out))) return fail(CTRAJ_EINVAL, "bad plane arguments");
  if (!std::isfinite(z_plane)) return fail(CTRAJ_EINVAL, "z_plane is not finite");
  for (int64_t k = 0; k < n_ids; ++k)
    if (ids[k] < 0 || ids[k] >= a->n) return fail(CTRAJ_EINVAL, "id %lld out of range", (long long)ids[k]);
  if (n_ids == 0) return CTRAJ_OK;
  Plan P;
  RunDev R;
  if ((st = prepare(c, a, P, R))) return st;
  for (int i = 0; i < P.n_el; ++i) P.lf[i].n_smem = 0;  // the replay reads tables from global memory
  const size_t ob = size_t(n_ids) * 8 * 8;
  if ((st = c->rec_rows.ensure(ob))) return st;
  if ((st = c->rec_ids.ensure(size_t(n_ids) * 8))) return st;
  CT_CUDA(cudaMemcpyAsync(c->rec_ids.p, ids, size_t(n_ids) * 8, cudaMemcpyHostToDevice, c->stream));
  const int threads = 128;
  const int grid = int((n_ids + threads - 1) / threads);
  if (a->precision == 32)
    k_plane<Mol32<true, true>, false><<<grid, threads, 0, c->stream>>>(P, R, c->rec_ids.as<int64_t>(), n_ids,
                                                                       z_plane, c->rec_rows.as<double>());
  else
    k_plane<Mol64<true>, true><<<grid, threads, 0, c->stream>>>(P, R, c->rec_ids.as<int64_t>(), n_ids, z_plane,
                                                                c->rec_rows.as<double>());
  CT_CUDA(cudaGetLastError());
  CT_CUDA(cudaMemcpyAsync(out, c->rec_rows.p, ob, cudaMemcpyDeviceToHost, c->stream));
  CT_CUDA(cudaStreamSynchronize(c->stream));
  return CTRAJ_OK;
}

int ctraj_run_ring(ctraj_context* c, const ctraj_run_args* a, const ctraj_ring* ring, ctraj_run_stats* stats) {
  if (!ring) return fail(CTRAJ_EINVAL, "ring is NULL");
  return run_impl(c, a, stats, ring);
}

int ctraj_record(ctraj_context* c, const ctraj_run_args* a, const int64_t* ids, int64_t n_ids,
                 int32_t stride, int32_t max_rows, double* rows, int32_t* row_count) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  int st = validate_run(c, a);
  if (st) return st;
  if (n_ids < 0 || (n_ids > 0 && (!ids || !rows || !row_count)) || stride < 1 || max_rows < 1)
    return fail(CTRAJ_EINVAL, "bad record arguments");
  for (int64_t k = 0; k < n_ids; ++k)
    if (ids[k] < 0 || ids[k] >= a->n) return fail(CTRAJ_EINVAL, "id %lld out of range", (long long)ids[k]);
  if (n_ids == 0) return CTRAJ_OK;
  Plan P;
  RunDev R;
  if ((st = prepare(c, a, P, R))) return st;
  for (int i = 0; i < P.n_el; ++i) P.lf[i].n_smem = 0;  // the replay reads tables from global memory
  const size_t rb = size_t(n_ids) * size_t(max_rows) * 10 * 8;
  if ((st = c->rec_rows.ensure(rb))) return st;
  if ((st = c->rec_ids.ensure(size_t(n_ids) * 8))) return st;
  if ((st = c->rec_count.ensure(align256(size_t(n_ids) * 4) + 256))) return st;
  unsigned* overflow = c->rec_count.as<unsigned>(align256(size_t(n_ids) * 4));
  CT_CUDA(cudaMemcpyAsync(c->rec_ids.p, ids, size_t(n_ids) * 8, cudaMemcpyHostToDevice, c->stream));
  CT_CUDA(cudaMemsetAsync(overflow, 0, 4, c->stream));
  const int threads = 128;
  const int grid = int((n_ids + threads - 1) / threads);
  if (a->precision == 32)
    k_record<Mol32<true, true>, false><<<grid, threads, 0, c->stream>>>(
        P, R, c->rec_ids.as<int64_t>(), n_ids, stride, max_rows, c->rec_rows.as<double>(),
        c->rec_count.as<int32_t>(), overflow);
  else
    k_record<Mol64<true>, true><<<grid, threads, 0, c->stream>>>(
        P, R, c->rec_ids.as<int64_t>(), n_ids, stride, max_rows, c->rec_rows.as<double>(),
        c->rec_count.as<int32_t>(), overflow);
  CT_CUDA(cudaGetLastError());
  unsigned ovf = 0;
  CT_CUDA(cudaMemcpyAsync(rows, c->rec_rows.p, rb, cudaMemcpyDeviceToHost, c->stream));
  CT_CUDA(cudaMemcpyAsync(row_count, c->rec_count.p, size_t(n_ids) * 4, cudaMemcpyDeviceToHost, c->stream));
  CT_CUDA(cudaMemcpyAsync(&ovf, overflow, 4, cudaMemcpyDeviceToHost, c->stream));
  CT_CUDA(cudaStreamSynchronize(c->stream));
  if (ovf) return fail(CTRAJ_EOVERFLOW, "%u molecules need more than max_rows = %d rows", ovf, max_rows);
  return CTRAJ_OK;
}

}  // extern "C"

