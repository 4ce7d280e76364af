// libctraj.so: the allocation-free run (ctraj_run_noalloc, declared in
// include/ctraj.h): the kernels of ctraj_run with every piece of scratch in one
// statically sized device array.
#include <mutex>

#include "engine.h"
#include "kernels.cuh"

using namespace ctraj;

// ============================================================================
// Allocation-free run (ctraj_run_noalloc): the same kernels as ctraj_run, with
// every piece of scratch in one statically sized device array.
// ============================================================================
namespace ctraj {
namespace {

// The scratch array.  Each GPU that loads this library holds it until exit.
// Host code must not use the name as a device address: it is a host-side
// stand-in; noalloc_scratch() looks up the real address per device.
static __device__ __align__(256) unsigned char g_noalloc_scratch[CTRAJ_NOALLOC_SCRATCH_BYTES];

// Layout: control words (queue counters, tallies, stats) | FP32 lens tables
// (kNaTables) | lens-entrant order (kNaOrder) | two lens queues (kNaQueues).
constexpr size_t kNaCtl = 0;
constexpr size_t kNaTables = 4096;
constexpr size_t kNaOrder = kNaTables + size_t(CTRAJ_NOALLOC_MAX_INTERVALS) * sizeof(float4);
constexpr size_t kNaQueues =
    kNaOrder + ((size_t(kOrderBuckets) + CTRAJ_NOALLOC_MAX_MOLECULES) * sizeof(unsigned) + 255) / 256 * 256;

// The array's device address differs between CUDA contexts (a non-primary
// context made with cuCtxCreate loads its own copy of the module, and a
// cudaDeviceReset replaces the primary context), so it is looked up once per
// context, keyed by the context's process-unique id (cuCtxGetId), with that
// context current.  The two driver functions are reached through the runtime
// (cudaGetDriverEntryPointByVersion): the library does not link libcuda.
struct NoallocSlot {
  unsigned long long ctx_id;
  void* ptr;
};
constexpr int kNoallocSlots = 64;
std::mutex g_noalloc_mu;
NoallocSlot g_noalloc_slot[kNoallocSlots] = {};
int g_noalloc_next = 0;
using CtxGetCurrentFn = int (*)(void**);
using CtxGetIdFn = int (*)(void*, unsigned long long*);
CtxGetCurrentFn g_ctx_current = nullptr;
CtxGetIdFn g_ctx_id = nullptr;

int noalloc_driver_fns() {
  if (g_ctx_current && g_ctx_id) return CTRAJ_OK;
  void* f0 = nullptr;
  void* f1 = nullptr;
  cudaDriverEntryPointQueryResult q0 = cudaDriverEntryPointSymbolNotFound, q1 = cudaDriverEntryPointSymbolNotFound;
  CT_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 12000, cudaEnableDefault, &q0));
  CT_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1));
  if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
    return fail(CTRAJ_ECUDA, "the CUDA driver does not provide cuCtxGetCurrent / cuCtxGetId");
  g_ctx_current = reinterpret_cast<CtxGetCurrentFn>(f0);
  g_ctx_id = reinterpret_cast<CtxGetIdFn>(f1);
  return CTRAJ_OK;
}

// Device address of the scratch array in the calling thread's current
// context: cudaGetSymbolAddress on the first call in that context (which
// also loads the module there), the cached address afterwards.
int noalloc_scratch(char** out) {
  int dev = 0;
  CT_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  int st = noalloc_driver_fns();
  if (st) return st;
  void* ctx = nullptr;
  if (g_ctx_current(&ctx) != 0) return fail(CTRAJ_ECUDA, "cuCtxGetCurrent failed");
  if (!ctx) {  // no context current yet: make the device's primary context current
    CT_CUDA(cudaSetDevice(dev));
    if (g_ctx_current(&ctx) != 0 || !ctx) return fail(CTRAJ_ECUDA, "no CUDA context on device %d", dev);
  }
  unsigned long long id = 0;
  if (g_ctx_id(ctx, &id) != 0) return fail(CTRAJ_ECUDA, "cuCtxGetId failed");
  for (const NoallocSlot& s : g_noalloc_slot)
    if (s.ptr && s.ctx_id == id) {
      *out = static_cast<char*>(s.ptr);
      return CTRAJ_OK;
    }
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) return fail(CTRAJ_ECUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
  g_noalloc_slot[g_noalloc_next] = NoallocSlot{id, p};  // the oldest context's entry is dropped
  g_noalloc_next = (g_noalloc_next + 1) % kNoallocSlots;
  *out = static_cast<char*>(p);
  return CTRAJ_OK;
}

int noalloc_check_table(const ctraj_force_table& t, int k) {
  if (t.kind == CTRAJ_TABLE_MESH) {
    if (t.n_knots < 1 || !t.knots || !t.values) return fail(CTRAJ_EINVAL, "table %d: mesh needs at least one cell", k);
    for (int j = 0; j < t.n_knots; ++j)
      if (!std::isfinite(t.knots[j]) || !std::isfinite(t.values[j]))
        return fail(CTRAJ_EINVAL, "table %d: cell %d is not finite", k, j);
    return CTRAJ_OK;
  }
  if (t.n_knots < 2 || !t.knots) return fail(CTRAJ_EINVAL, "table %d needs at least 2 knots", k);
  if (t.kind == CTRAJ_TABLE_STARK_SPLINE && !t.coef) return fail(CTRAJ_EINVAL, "table %d: no coef", k);
  if (t.kind == CTRAJ_TABLE_RADIAL_LINEAR && !t.values) return fail(CTRAJ_EINVAL, "table %d: no values", k);
  if (t.kind != CTRAJ_TABLE_STARK_SPLINE && t.kind != CTRAJ_TABLE_RADIAL_LINEAR)
    return fail(CTRAJ_EINVAL, "table %d: unknown kind %d", k, t.kind);
  const double h = (t.knots[t.n_knots - 1] - t.knots[0]) / double(t.n_knots - 1);
  if (!(h > 0)) return fail(CTRAJ_EINVAL, "table %d: knots must ascend", k);
  for (int j = 1; j < t.n_knots; ++j)
    if (std::fabs((t.knots[j] - t.knots[j - 1]) - h) > 1e-6 * h)
      return fail(CTRAJ_EINVAL, "table %d: knots must be uniformly spaced", k);
  return CTRAJ_OK;
}

// Host-side checks of the elements' tables, before any CUDA call: table ids,
// mesh shapes, lens field orders, and that the FP32 tables of all lenses and
// meshes fit the scratch's CTRAJ_NOALLOC_MAX_INTERVALS float4 entries.
int noalloc_check_tables(const ctraj_element* el, int n_el, const ctraj_force_table* tabs, int n_tab) {
  size_t total = 0;
  for (int i = 0; i < n_el; ++i) {
    const ctraj_element& e = el[i];
    if (e.type != CTRAJ_ELECTROSTATIC_LENS && e.type != CTRAJ_HONEYCOMB) continue;
    if (e.table < 0 || e.table >= n_tab) return fail(CTRAJ_ESTATE, "element %d uses table %d, not given", i, e.table);
    const ctraj_force_table& t = tabs[e.table];
    if (e.type == CTRAJ_HONEYCOMB) {
      int st = check_honeycomb(e, i, t.kind, t.n_knots);
      if (st) return st;
      total += size_t(t.n_knots);
    } else {
      if (t.kind == CTRAJ_TABLE_MESH) return fail(CTRAJ_EINVAL, "lens element %d: table %d is a mesh table", i, e.table);
      if (t.kind == CTRAJ_TABLE_STARK_SPLINE && e.field_order != 1 && e.field_order != 2)
        return fail(CTRAJ_EINVAL, "lens element %d: field_order must be 1 or 2", i);
      const bool lin = stark_linear(t.kind, t.n_knots, t.knots, t.coef, e);
      total += size_t(t.n_knots - 1) * (lin ? 2 : 1);
    }
  }
  if (total > size_t(CTRAJ_NOALLOC_MAX_INTERVALS))
    return fail(CTRAJ_EINVAL, "lens and mesh tables need %zu float4 entries: the scratch holds at most %d",
                total, CTRAJ_NOALLOC_MAX_INTERVALS);
  return CTRAJ_OK;
}

// Plan and FP32 lens tables (written into the scratch through a small stack
// buffer: nothing is allocated on the host heap either).  The tables were
// checked by noalloc_check_tables.
int noalloc_plan(const ctraj_element* el, int n_el, int n_labels, const ctraj_force_table* tabs,
                 int n_tab, const ctraj_run_args* a, float4* dev_tables, cudaStream_t s, Plan& P) {
  std::memset(&P, 0, sizeof P);
  P.n_el = n_el;
  P.n_labels = n_labels;
  P.first_lens = n_el;
  P.g = a->g;
  P.gf = float(a->g);
  size_t offset = 0;
  float4 buf[256];
  for (int i = 0; i < n_el; ++i) {
    const ctraj_element& e = el[i];
    P.el[i] = e;
    ElemF& f = P.ef[i];
    f.gap = i > 0 ? float(e.z0 - el[i - 1].z1) : 0.f;
    f.len = float(e.z1 - e.z0);
    if (e.type == CTRAJ_CIRCULAR_APERTURE || e.type == CTRAJ_ELECTROSTATIC_LENS) {
      const double h = e.p[0] * 0.5;
      f.c[0] = float(h * h);
      f.c[1] = float(h);
    } else if (e.type == CTRAJ_RECTANGULAR_APERTURE) {
      for (int k = 0; k < 4; ++k) f.c[k] = float(e.p[k]);
    } else if (e.type == CTRAJ_FIELD_PLATES) {
      f.c[0] = float(e.p[0]);
      f.c[1] = float(e.p[1]);
    } else if (e.type == CTRAJ_HONEYCOMB) {
      honeycomb_constants(e, f);
    }
    if (e.type != CTRAJ_ELECTROSTATIC_LENS && e.type != CTRAJ_HONEYCOMB) continue;
    const ctraj_force_table& t = tabs[e.table];
    if (e.type == CTRAJ_HONEYCOMB) {  // cell centres (x, y, 0, 0)
      for (int j0 = 0; j0 < t.n_knots; j0 += 256) {
        const int m = std::min(256, t.n_knots - j0);
        for (int j = 0; j < m; ++j)
          buf[j] = make_float4(float(t.knots[j0 + j]), float(t.values[j0 + j]), 0.f, 0.f);
        CT_CUDA(cudaMemcpyAsync(dev_tables + offset + j0, buf, m * sizeof(float4), cudaMemcpyHostToDevice, s));
      }
      P.lf[i].q = dev_tables + offset;
      P.lf[i].n_int = t.n_knots;
      P.lf[i].cols = int(e.p[1]);
      offset += size_t(t.n_knots);
      continue;
    }
    if (P.first_lens == n_el) P.first_lens = i;
    const int n_int = t.n_knots - 1;
    const bool lin = stark_linear(t.kind, t.n_knots, t.knots, t.coef, e);
    const int entries = lin ? 2 * n_int : n_int;  // float4
    const double x0 = t.knots[0], h = (t.knots[t.n_knots - 1] - t.knots[0]) / double(n_int);
    const double alpha = e.p[6], mass = e.p[5];
    const double kappa = e.field_order == 1 ? alpha / mass : 2.0 * alpha / mass;
    for (int j0 = 0; j0 < entries; j0 += 256) {
      const int m = std::min(256, entries - j0);
      for (int j = 0; j < m; ++j) {
        const int k = j0 + j;
        if (t.kind == CTRAJ_TABLE_RADIAL_LINEAR) {
          buf[j] = make_float4(float(t.values[k]), float(t.values[k + 1] - t.values[k]), 0.f, 0.f);
        } else {
          const int iv = lin ? k / 2 : k;
          const double* ck = &t.coef[size_t(iv) * 4];
          const double qa = -kappa * ck[2], qb = -kappa * 2.0 * ck[1] * h, qc = -kappa * 3.0 * ck[0] * h * h;
          buf[j] = lin ? stark_pieces(qa, qb, qc, k % 2) : make_float4(float(qa), float(qb), float(qc), 0.f);
        }
      }
      // pageable source: the call returns once buf has been staged, so buf can be refilled
      CT_CUDA(cudaMemcpyAsync(dev_tables + offset + j0, buf, m * sizeof(float4), cudaMemcpyHostToDevice, s));
    }
    LensF& L = P.lf[i];
    L.q = dev_tables + offset;
    L.n_int = entries;
    L.n_smem = entries <= (lin ? kMaxStagedLinear : kMaxStagedIntervals) ? entries : 0;
    L.outward = 0;  // entrants ordered by step count alone
    if (t.kind == CTRAJ_TABLE_RADIAL_LINEAR) {
      L.force = kForceRadial;
      L.beta = float(1.0 / h);
      L.s0 = float(x0 / h);
      L.r_max = float(t.knots[t.n_knots - 1]);
    } else {
      L.force = lin ? kForceStark2Lin : (e.field_order == 1 ? kForceStark1 : kForceStark2);
      const double scale = lin ? double(kLinearPieces) : 1.0;  // pieces
      L.beta = float(scale * alpha / h);
      L.s0 = float(scale * x0 / h);
      L.r_max = INFINITY;
    }
    offset += size_t(entries);
  }
  return CTRAJ_OK;
}

// The launch sequence of launch_all (FP32), on the scratch's queues.
// *max_steps receives the largest lens step bound of any lens queue.
template <bool kOut>
int noalloc_launch(const Plan& P, const RunDev& R, Queue* q, unsigned* order_buf, cudaStream_t s,
                   int* launches, unsigned* max_steps) {
  int dev = 0, sms = 0;
  CT_CUDA(cudaGetDevice(&dev));
  CT_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t n = R.n;
  if (n > 0) {
    int st = launch_front(P, R, q[0], n, 32, kOut, kModePlain, kThreads, sms, 4, s);
    if (st) return st;
    ++*launches;
  }
  int cur = 0, nxt = 1;
  for (int i = 0; i < P.n_el && n > 0; ++i) {
    if (P.el[i].type != CTRAJ_ELECTROSTATIC_LENS) continue;
    unsigned ctl[2] = {0, 0};  // the queue's count and largest step bound
    CT_CUDA(cudaMemcpyAsync(ctl, q[cur].count, sizeof ctl, cudaMemcpyDeviceToHost, s));
    CT_CUDA(cudaStreamSynchronize(s));
    const unsigned count = ctl[0];
    *max_steps = std::max(*max_steps, ctl[1]);
    if (count == 0) break;
    CT_CUDA(cudaMemsetAsync(q[nxt].count, 0, kCtlWords * sizeof(unsigned), s));
    // the persistent pass finishes every molecule: nothing stays inside the lens
    int st = enqueue_persistent(kOut, kModePlain, P, R, i, q[cur], q[nxt], order_buf, sms, 256, kPersistService, s,
                                launches, kPersistThreads, 1);
    if (st) return st;
    std::swap(cur, nxt);
  }
  return CTRAJ_OK;
}

}  // namespace
}  // namespace ctraj

extern "C" int ctraj_run_noalloc(const ctraj_element* el, int32_t n_el, int32_t n_labels,
                                 const ctraj_force_table* tabs, int32_t n_tab,
                                 const ctraj_run_args* a, void* stream, ctraj_run_stats* stats) {
  if (!a) return fail(CTRAJ_EINVAL, "args is NULL");
  if (a->precision != 32) return fail(CTRAJ_EINVAL, "ctraj_run_noalloc supports precision 32 only");
  if (a->n < 0 || a->n > CTRAJ_NOALLOC_MAX_MOLECULES)
    return fail(CTRAJ_EINVAL, "n = %lld: ctraj_run_noalloc takes at most %d molecules per call",
                (long long)a->n, CTRAJ_NOALLOC_MAX_MOLECULES);
  if (a->ic_mode == CTRAJ_IC_HOST) return fail(CTRAJ_EINVAL, "ctraj_run_noalloc needs device-memory initial conditions");
  if (a->ic_mode == CTRAJ_IC_DEVICE_DRAW) {
    if (a->xdist.kind != CTRAJ_DIST_GAUSSIAN_POSITION && a->xdist.kind != CTRAJ_DIST_DISC_POSITION)
      return fail(CTRAJ_EINVAL, "unknown position distribution kind %d", a->xdist.kind);
    if (a->vdist.kind != CTRAJ_DIST_GAUSSIAN_VELOCITY)
      return fail(CTRAJ_EINVAL, "unknown velocity distribution kind %d", a->vdist.kind);
  } else if (a->ic_mode == CTRAJ_IC_DEVICE) {
    if (!a->ics && a->n > 0) return fail(CTRAJ_EINVAL, "ics is NULL");
  } else {
    return fail(CTRAJ_EINVAL, "unknown ic_mode %d", a->ic_mode);
  }
  if (a->out_mode == CTRAJ_OUT_HOST) return fail(CTRAJ_EINVAL, "ctraj_run_noalloc writes per-molecule outputs to device memory only");
  if (a->out_mode != CTRAJ_OUT_NONE && a->out_mode != CTRAJ_OUT_DEVICE) return fail(CTRAJ_EINVAL, "bad out_mode");
  if (!a->counts) return fail(CTRAJ_EINVAL, "counts is NULL");
  if (n_el < 0 || n_el > CTRAJ_MAX_ELEMENTS || (n_el > 0 && !el)) return fail(CTRAJ_EINVAL, "bad elements");
  if (n_labels < 0 || n_labels > CTRAJ_MAX_LABELS) return fail(CTRAJ_EINVAL, "n_labels %d out of range", n_labels);
  if (n_tab < 0 || n_tab > CTRAJ_MAX_TABLES || (n_tab > 0 && !tabs)) return fail(CTRAJ_EINVAL, "bad tables");
  for (int i = 0; i < n_el; ++i) {
    const ctraj_element& e = el[i];
    if (e.type < CTRAJ_CIRCULAR_APERTURE || e.type > CTRAJ_HONEYCOMB)
      return fail(CTRAJ_EINVAL, "element %d: unknown type %d", i, e.type);
    if (e.label < -1 || e.label >= n_labels || e.label_inside < -1 || e.label_inside >= n_labels)
      return fail(CTRAJ_EINVAL, "element %d: label out of range", i);
    if (i > 0 && e.z0 < el[i - 1].z0) return fail(CTRAJ_EINVAL, "elements are not sorted by z0 (element %d)", i);
  }
  for (int k = 0; k < n_tab; ++k) {
    int st = noalloc_check_table(tabs[k], k);
    if (st) return st;
  }
  int st = noalloc_check_tables(el, n_el, tabs, n_tab);
  if (st) return st;
  char* scratch = nullptr;
  if ((st = noalloc_scratch(&scratch))) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t cap = CTRAJ_NOALLOC_MAX_MOLECULES;
  const size_t qb = queue_bytes(cap, 32);
  if (kNaQueues + 2 * qb > CTRAJ_NOALLOC_SCRATCH_BYTES) return fail(CTRAJ_ENOMEM, "scratch layout too large");
  Plan P;
  if ((st = noalloc_plan(el, n_el, n_labels, tabs, n_tab, a, reinterpret_cast<float4*>(scratch + kNaTables), s, P)))
    return st;
  unsigned* ctl = reinterpret_cast<unsigned*>(scratch + kNaCtl);
  unsigned long long* counts = reinterpret_cast<unsigned long long*>(scratch + kNaCtl + 256);
  unsigned long long* dstats = reinterpret_cast<unsigned long long*>(scratch + kNaCtl + 256 + 8 * (CTRAJ_MAX_LABELS + 1));
  // queues are handed over in DevBuf form so the same layout code places the arrays
  Queue q[2];
  for (int k = 0; k < 2; ++k) {
    DevBuf view;
    view.p = scratch + kNaQueues + size_t(k) * qb;
    view.bytes = qb;
    layout_queue(&view, cap, 32, ctl + kCtlWords * k, &q[k]);
    view.p = nullptr;  // a view: nothing to free
  }
  CT_CUDA(cudaMemsetAsync(scratch + kNaCtl, 0, 4096, s));  // counters, tallies and stats start at zero
  RunDev R;
  std::memset(&R, 0, sizeof R);
  R.n = a->n;
  R.seed = a->seed;
  R.key = philox_key(a->seed);
  R.offset = a->offset;
  R.ic_mode = a->ic_mode;
  R.xd = a->xdist;
  R.vd = a->vdist;
  R.ics = a->ics;
  if (a->ic_mode == CTRAJ_IC_DEVICE_DRAW) {
    const double zd = a->xdist.kind == CTRAJ_DIST_DISC_POSITION ? a->xdist.p[1] : a->xdist.p[2];
    R.gap0f = P.n_el > 0 ? float(P.el[0].z0 - zd) : 0.f;
  }
  R.counts = counts;
  R.stats = dstats;
  const bool out = a->out_mode == CTRAJ_OUT_DEVICE;
  if (out) {
    R.out_label = a->out_label;
    R.out_rows = a->out_rows;
    R.out_margin = a->out_margin;
    R.out_final = a->out_final;
  }
  int launches = 0;
  unsigned max_steps = 0;
  unsigned* order_buf = reinterpret_cast<unsigned*>(scratch + kNaOrder);
  st = out ? noalloc_launch<true>(P, R, q, order_buf, s, &launches, &max_steps)
           : noalloc_launch<false>(P, R, q, order_buf, s, &launches, &max_steps);
  if (st) return st;
  unsigned long long hc[CTRAJ_MAX_LABELS + 1], hs[kStatCount];
  CT_CUDA(cudaMemcpyAsync(hc, counts, sizeof hc, cudaMemcpyDeviceToHost, s));
  CT_CUDA(cudaMemcpyAsync(hs, dstats, sizeof hs, cudaMemcpyDeviceToHost, s));
  CT_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k <= n_labels; ++k) a->counts[k] = int64_t(hc[k]);
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->molecules = a->n;
    stats->molecule_steps = int64_t(hs[kStatSteps]);
    stats->lens_steps = int64_t(hs[kStatLensSteps]);
    stats->edge_band = out ? int64_t(hs[kStatEdgeBand]) : -1;
    stats->table_range = int64_t(hs[kStatTableRange]);
    stats->bad_steps = int64_t(hs[kStatBadSteps]);
    stats->kernels = launches;
    stats->max_lens_steps = int32_t(max_steps);
    for (int i = 0; i < P.n_el; ++i)
      stats->linear_tables += P.el[i].type == CTRAJ_ELECTROSTATIC_LENS && P.lf[i].force == kForceStark2Lin;
  }
  if (hs[kStatRangeError])
    return fail(CTRAJ_ERANGE, "%llu molecules looked up the lens table above its last knot", hs[kStatRangeError]);
  if (hs[kStatBadSteps])
    return fail(CTRAJ_ESTEPS, "%llu molecules have a non-finite or oversize lens step count", hs[kStatBadSteps]);
  return CTRAJ_OK;
}
