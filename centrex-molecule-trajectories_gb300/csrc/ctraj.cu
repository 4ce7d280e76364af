// libctraj.so: C ABI of the GB300 trajectory engine (declared in include/ctraj.h).
//
// A context owns one CUDA stream (or borrows the caller's), the device copies
// of the beamline's force tables, the FP32 lens tables derived from them, and
// grow-only work buffers (lens queues, injected initial conditions,
// per-molecule outputs).  ctraj_run enqueues k_front and the chunked lens
// kernels and copies the per-label counts back; nothing is allocated on a
// repeated run of the same or a smaller size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <system_error>
#include <thread>
#include <type_traits>
#include <vector>

#include "ctraj.h"
#include "adjoint.cuh"
#include "kernels.cuh"

namespace ctraj {
namespace {

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

#define CT_CUDA(call)                                                                   \
  do {                                                                                  \
    cudaError_t e_ = (call);                                                            \
    if (e_ != cudaSuccess) return fail(CTRAJ_ECUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  // headroom_pct: when growing, allocate that much more, for buffers sized by
  // a count that varies from run to run (a cudaFree/cudaMalloc in a run
  // synchronizes the device)
  int ensure(size_t want, size_t headroom_pct = 0) {
    if (want <= bytes) return CTRAJ_OK;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    want += want / 100 * headroom_pct;
    cudaError_t e = cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(CTRAJ_ENOMEM, "cudaMalloc(%zu): %s", want, cudaGetErrorString(e));
    }
    bytes = want;
    return CTRAJ_OK;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as(size_t offset_bytes = 0) const {
    return reinterpret_cast<T*>(static_cast<char*>(p) + offset_bytes);
  }
};

struct HostTable {
  int kind = 0;
  int n = 0;
  std::vector<double> knots, coef, values;
  DevBuf dev;  // knots | coef | values
  bool uploaded = false;
};

}  // namespace
}  // namespace ctraj

using namespace ctraj;

struct ctraj_context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<ctraj_element> elements;
  int n_labels = 0;
  bool have_beamline = false;
  HostTable tables[CTRAJ_MAX_TABLES];
  DevBuf lens_tables;           // FP32 lens tables, one region per lens element
  bool lens_tables_dirty = true;
  std::vector<size_t> lens_offset;
  std::vector<int> lens_n_int, lens_n_smem;
  DevBuf queue[3];              // lens queues: current chunk, continuation, next lens
  DevBuf qctl;                  // queue counters (2 x unsigned per queue) + counts + stats
  DevBuf ics;
  DevBuf outs;
  DevBuf rec_rows, rec_ids, rec_count;
  unsigned* host_max = nullptr; // pinned: largest remaining lens step count of a queue
  DevBuf chunk_ctl;             // (count, max_steps) of the queue each lens chunk writes
  DevBuf rec_stage;             // ring recording: staged records of the recorded lens
  DevBuf ring_ent;              // ring recording: molecules stopped by the entrance test
  DevBuf lens_order;            // persistent lens pass: bucket counts | entrant order
  DevBuf sweep_order;           // persistent sweep: per table bucket counts | entrant order
  int chunk = 64;               // RK4 steps of the first lens chunk (compaction interval)
  int chunk_growth = 200;       // percent: each chunk's length relative to the previous
  int chunk_max = 1024;         // longest chunk
  int front_waves = 4;          // k_front grid in units of resident CTAs
  int lens_mode = CTRAJ_LENS_PERSISTENT;  // FP32 lens pass
  int lens_interval = 256;      // persistent mode: steps between CTA compactions
  int front_threads = 256;      // k_front block size
  int batch_group = 4;          // ctraj_run_batch: runs sharing one lens pass
  int lens_threads = 512;       // persistent FP32 lens pass: molecule lanes per CTA
  int lens_molecules = 1;       // persistent FP32 lens pass: molecules per thread
  unsigned run_max_steps = 0;   // largest lens queue step bound of the last run
  bool timing = false;
  // before front, after front, before the first lens chunk, after the last one
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // bumped by every call that changes what a captured sweep graph depends on
  uint64_t generation = 0;
  // batched sweeps (ctraj_run_sweep), set up on first use
  DevBuf sweep_tables;          // unscaled FP32 Stark tables, one region per table used
  DevBuf sweep_cfg;             // per-configuration arrays and counts
  DevBuf sweep_ctl;             // queue counters, chunk counters, totals, stats
  DevBuf sweep_queue[2 * CTRAJ_MAX_TABLES];
  // soft transmission (ctraj_soft_transmission)
  DevBuf soft_table, soft_queue, soft_ckpt, soft_ctl, soft_contrib, soft_seg;
  unsigned long long* sweep_host = nullptr;  // pinned: per-configuration counts, totals, stats
  size_t sweep_host_words = 0;
  cudaStream_t side[CTRAJ_MAX_TABLES] = {};
  cudaEvent_t fork = nullptr, join[CTRAJ_MAX_TABLES] = {};
  cudaGraphExec_t sweep_exec = nullptr;
  std::vector<char> sweep_key;  // inputs the captured graph was built from
  int sweep_launches = 0;
  // pipelined batches (ctraj_run_batch): the second lane's context, a copy of
  // this one's beamline, tables and tuning as of generation peer_generation
  ctraj_context* peer = nullptr;
  uint64_t peer_generation = ~uint64_t(0);
  DevBuf l2_flush;              // scratch written before each run of a batch
  cudaEvent_t batch_ev = nullptr;
  // grouped batches: per-run counts and stats (device and pinned host), the
  // host initial conditions of a group's runs
  DevBuf group_ctl;
  unsigned long long* group_host = nullptr;
  size_t group_host_words = 0;
  DevBuf group_ics;
};

namespace ctraj {
namespace {

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

constexpr int kMaxStagedIntervals = 6144;  // 96 KiB of float4 per CTA
// a kForceStark2Lin table (two float4 of pieces per knot interval) is staged
// up to 128 KiB: with the persistent pass's 40 KiB of swap slots one CTA per SM
constexpr int kMaxStagedLinear = 8192;
constexpr int kMaxChunks = 16384;          // lens chunks per lens (CTRAJ_MAX_LENS_STEPS / 1024 < this)

// Queue layout inside one buffer of capacity cap (SoA, each array 256-byte
// aligned so a warp's 32 consecutive entries are whole 128-byte lines).
// Returns the bytes used; with b == nullptr only sizes the layout.
size_t layout_queue(const DevBuf* b, size_t cap, int precision, unsigned* ctl, Queue* q,
                    bool with_cfg = false) {
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

size_t queue_bytes(size_t cap, int precision, bool with_cfg = false) {
  return layout_queue(nullptr, cap, precision, nullptr, nullptr, with_cfg);
}

// FP32 Stark tables of field order 2 reach the lens kernels as linear pieces
// on quarter intervals (kForceStark2Lin: one 8-byte lookup instead of a
// 16-byte quadratic) when both hold:
//  * accuracy: linear interpolation of the quadratic w(u) = a + b u + c u^2
//    of an interval over its quarters departs from it by at most |c| / 64;
//    that must stay below kLinearTolerance of the largest |w| (the 4096-knot
//    hexapole table: 4.0e-7);
//  * coverage: the table starts at or below |E| = 0 and reaches |E| at
//    kLinearCover times the bore radius, so a molecule inside the bore (and
//    every RK4 stage point of its next step) looks up inside the table, where
//    the quadratic form would need no extrapolation either; beyond the last
//    knot a piece extrapolates linearly;
// and the pieces (2 float4 per interval) fit the 128 KiB staging limit.
// Otherwise the 16-byte quadratic (kForceStark2), exact per interval.
constexpr double kLinearTolerance = 1e-6;
constexpr double kLinearCover = 1.2;
constexpr int kLinearPieces = 4;  // per knot interval

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

template <class KernelT>
int blocks_per_sm(KernelT k, int threads, size_t smem) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, threads, smem) != cudaSuccess || b < 1) b = 1;
  return b;
}

// k_front over n molecules into queue Q: threads per block, a grid of
// `waves` x resident CTAs (or fewer), the staging area for lens entrants in
// dynamic shared memory.
template <class M, bool kOut, int kMode>
int launch_front(const Plan& P, const RunDev& R, const Queue& Q, int64_t n, int threads, int sms, int waves,
                 cudaStream_t s) {
  auto kf = k_front<M, kOut, kMode>;
  const size_t smem = front_smem<M>(threads);
  CT_CUDA(cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  const int bps = blocks_per_sm(kf, threads, smem);
  const int64_t want = (n + threads - 1) / threads;
  const int grid = int(std::min<int64_t>(want, int64_t(bps) * sms * waves));
  kf<<<grid, threads, smem, s>>>(P, R, Q);
  CT_CUDA(cudaGetLastError());
  return CTRAJ_OK;
}

// The lens kernel for lens element i: FP32 is specialised on the force law,
// FP64 evaluates the reference's force code for every table kind.
using LensKernel = void (*)(const Plan, const RunDev, const int, const Queue, const Queue,
                            const Queue, const int, const LensArgs);

template <bool kOut, bool kStaged, bool kRing>
LensKernel lens_kernel32(int force) {
  using M = Mol32<kOut, false>;
  switch (force) {
    case kForceStark2: return k_lens_chunk<M, kOut, kForceStark2, false, kStaged, false, kRing>;
    case kForceStark2Lin: return k_lens_chunk<M, kOut, kForceStark2Lin, false, kStaged, false, kRing>;
    case kForceStark1: return k_lens_chunk<M, kOut, kForceStark1, false, kStaged, false, kRing>;
    default: return k_lens_chunk<M, kOut, kForceRadial, false, kStaged, false, kRing>;
  }
}

template <bool k64, bool kOut, bool kRing = false>
LensKernel lens_kernel(int force, bool staged) {
  if (k64) return k_lens_chunk<Mol64<false>, kOut, 0, true, false>;
  return staged ? lens_kernel32<kOut, true, kRing>(force) : lens_kernel32<kOut, false, kRing>(force);
}

// The persistent FP32 lens pass of lens element i over queue Qin: order the
// entrants longest first into `order_buf` (kOrderBuckets + the queue's
// entries), then one k_lens_persist launch, one CTA per SM.  kMode: plain,
// ring recording or grouped batch.  lanes: molecules per CTA (tuning
// lens_threads), mpt: molecules per thread (tuning lens_molecules), so the CTA
// has lanes / mpt threads.  Compiled for the staged-table plain and batch
// passes without per-molecule outputs (the throughput path): 512, 768 or
// 1024 lanes at one molecule per thread, and for the hexapole Stark forms
// also at two; every other pass (and setting) runs 512 threads x 1.
using PersistKernel = void (*)(const Plan, const RunDev, const int, const Queue, const Queue, const LensArgs,
                               const unsigned*, const int);

template <bool kOut, int F, bool kStaged, int kMode>
PersistKernel persist_kernel(int lanes, int mpt, int* threads, int* used_mpt) {
  using M = Mol32<kOut, false>;
  *used_mpt = 1;
  if constexpr (!kOut && kStaged && (kMode == kModePlain || kMode == kModeBatch)) {
    if constexpr (F == kForceStark2 || F == kForceStark2Lin) {
      if (mpt == 2) {
        *used_mpt = 2;
        *threads = lanes / 2;
        if (lanes == 1024) return k_lens_persist<M, kOut, F, kStaged, kMode, 512, 2>;
        if (lanes == 768) return k_lens_persist<M, kOut, F, kStaged, kMode, 384, 2>;
        *threads = 256;
        return k_lens_persist<M, kOut, F, kStaged, kMode, 256, 2>;
      }
    }
    if (lanes == 1024) {
      *threads = 1024;
      return k_lens_persist<M, kOut, F, kStaged, kMode, 1024>;
    }
    if (lanes == 768) {
      *threads = 768;
      return k_lens_persist<M, kOut, F, kStaged, kMode, 768>;
    }
  }
  *threads = kPersistThreads;
  return k_lens_persist<M, kOut, F, kStaged, kMode, kPersistThreads>;
}

template <bool kOut, int F, int kMode>
PersistKernel persist_kernel(bool staged, int lanes, int mpt, int* threads, int* used_mpt) {
  return staged ? persist_kernel<kOut, F, true, kMode>(lanes, mpt, threads, used_mpt)
                : persist_kernel<kOut, F, false, kMode>(lanes, mpt, threads, used_mpt);
}

template <bool kOut, int kMode = kModePlain>
int enqueue_persistent(const Plan& P, const RunDev& R, int i, const Queue& Qin, const Queue& Qnext,
                       unsigned* order_buf, int sms, int interval, cudaStream_t s, int* launches,
                       int lanes = kPersistThreads, int mpt = 1) {
  const bool staged = P.lf[i].n_smem > 0;
  int kt = kPersistThreads, km = 1;
  PersistKernel k;
  switch (P.lf[i].force) {
    case kForceStark2: k = persist_kernel<kOut, kForceStark2, kMode>(staged, lanes, mpt, &kt, &km); break;
    case kForceStark2Lin: k = persist_kernel<kOut, kForceStark2Lin, kMode>(staged, lanes, mpt, &kt, &km); break;
    case kForceStark1: k = persist_kernel<kOut, kForceStark1, kMode>(staged, lanes, mpt, &kt, &km); break;
    default: k = persist_kernel<kOut, kForceRadial, kMode>(staged, lanes, mpt, &kt, &km); break;
  }
  const size_t smem =
      (staged ? size_t(P.lf[i].n_int) * sizeof(float4) : 0) + size_t(kt) * size_t(km) * sizeof(SwapSlot);
  CT_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  unsigned* hist = order_buf;
  unsigned* order = hist + kOrderBuckets;
  CT_CUDA(cudaMemsetAsync(hist, 0, kOrderBuckets * sizeof(unsigned), s));
  k_order_count<<<sms, kOrderThreads, 0, s>>>(P, i, Qin, hist);
  k_order_scan<<<1, kOrderBuckets, 0, s>>>(hist);
  k_order_place<<<sms, kOrderThreads, 0, s>>>(P, i, Qin, hist, order);
  k<<<sms, kt, smem, s>>>(P, R, i, Qin, Qnext, lens_args(P, i, true), order, interval);
  CT_CUDA(cudaGetLastError());
  *launches += 4;
  return CTRAJ_OK;
}

template <bool kOut, int kMode = kModePlain>
int launch_persistent(ctraj_context* c, const Plan& P, const RunDev& R, int i, const Queue& Qin, const Queue& Qnext,
                      unsigned count, int* launches) {
  int st = c->lens_order.ensure((size_t(kOrderBuckets) + count) * sizeof(unsigned), 25);
  if (st) return st;
  return enqueue_persistent<kOut, kMode>(P, R, i, Qin, Qnext, c->lens_order.as<unsigned>(), c->sm_count,
                                         c->lens_interval, c->stream, launches, c->lens_threads,
                                         c->lens_molecules);
}

// k_front, then for each lens: read the lens queue's size and largest
// remaining step count (one small device-to-host copy), and launch
// ceil(max / chunk) chunk kernels that ping-pong between two queues while
// molecules leaving the lens collect in a third for the next lens.
// *left receives the molecules still in a lens afterwards (always 0).
template <bool k64, bool kOut, bool kRing = false>
int launch_all(ctraj_context* c, const Plan& P, const RunDev& R0, Queue* q, int* launches) {
  using MolT = typename std::conditional<k64, Mol64<false>, Mol32<kOut, false>>::type;
  RunDev R = R0;  // ring recording fills in the staging buffers once the lens count is known
  c->run_max_steps = 0;
  unsigned ring_slots = 0;
  const int64_t n = R.n;
  cudaStream_t s = c->stream;
  if (c->timing) CT_CUDA(cudaEventRecord(c->ev[0], s));
  if (n > 0) {
    int st = launch_front<MolT, kOut, kRing ? kModeRing : kModePlain>(P, R, q[0], n, c->front_threads, c->sm_count,
                                                                       c->front_waves, s);
    if (st) return st;
    ++*launches;
  }
  if (c->timing) CT_CUDA(cudaEventRecord(c->ev[1], s));
  bool started = false;
  int cur = 0, alt = 1, nxt = 2;
  for (int i = 0; i < P.n_el && n > 0; ++i) {
    if (P.el[i].type != CTRAJ_ELECTROSTATIC_LENS) continue;
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
    LensKernel kl = lens_kernel<k64, kOut, kRing>(P.lf[i].force, staged);
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
        int st = launch_persistent<kOut, kRing ? kModeRing : kModePlain>(c, P, R, i, q[cur], q[nxt], count, launches);
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
    k_ring_reserve<<<c->sm_count * 8, 256, 0, s>>>(R, ring_slots);
    CT_CUDA(cudaGetLastError());
    if constexpr (!k64) {
      k_ring_write<Mol32<false, false>><<<c->sm_count * 8, 256, 0, s>>>(P, R, ring_slots);
      CT_CUDA(cudaGetLastError());
    }
    *launches += 2;
  }
  if (c->timing) {
    if (!started) CT_CUDA(cudaEventRecord(c->ev[2], s));
    CT_CUDA(cudaEventRecord(c->ev[3], s));
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

}  // namespace
}  // namespace ctraj

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
      (t->lens_molecules != 1 && t->lens_molecules != 2))
    return fail(CTRAJ_EINVAL,
                "tuning out of range (chunk_first %d, chunk_growth %d, chunk_max %d, front_waves %d, lens_mode %d, "
                "lens_interval %d, front_threads %d, batch_group %d, lens_threads %d, lens_molecules %d)",
                t->chunk_first, t->chunk_growth, t->chunk_max, t->front_waves, t->lens_mode, t->lens_interval,
                t->front_threads, t->batch_group, t->lens_threads, t->lens_molecules);
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
  c->elements.assign(el, el + n_el);
  c->n_labels = n_labels;
  c->have_beamline = true;
  c->lens_tables_dirty = true;
  ++c->generation;
  return CTRAJ_OK;
}

int ctraj_set_force_table(ctraj_context* c, int32_t id, const ctraj_force_table* t) {
  if (!c || !t) return fail(CTRAJ_EINVAL, "NULL argument");
  if (id < 0 || id >= CTRAJ_MAX_TABLES) return fail(CTRAJ_EINVAL, "table id %d out of range", id);
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
    if ((st = launch_front<Mol32<false, false>, false, kModeBatch>(P, R[j], q[0], a[j].n, c->front_threads,
                                                                  c->sm_count, c->front_waves, s)))
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
  for (int i = 0; i < P.n_el && total > 0; ++i) {
    if (P.el[i].type != CTRAJ_ELECTROSTATIC_LENS) continue;
    CT_CUDA(cudaMemcpyAsync(c->host_max, q[cur].count, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CT_CUDA(cudaStreamSynchronize(s));
    const unsigned count = c->host_max[0];
    if (count == 0) break;
    if (timing && !started) CT_CUDA(cudaEventRecord(c->ev[2], s));
    started = true;
    CT_CUDA(cudaMemsetAsync(q[nxt].count, 0, kCtlWords * sizeof(unsigned), s));
    if ((st = launch_persistent<false, kModeBatch>(c, P, Rg, i, q[cur], q[nxt], count, &launches))) return st;
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

// ============================================================================
// Batched sweep (ctraj_run_sweep): one front launch over every configuration's
// molecules, then per Stark table one fixed chunk sequence on its own stream;
// optionally captured once as a CUDA graph.
// ============================================================================
namespace ctraj {
namespace {

constexpr int kMaxSweepChunks = 1024;  // lens chunks per table, the unbounded last one included

// sweep_ctl: entrance-queue words per table, then output-queue words per
// (table, chunk).
constexpr size_t kSwChunkCtl = 4096;
constexpr size_t kSwCtlBytes =
    kSwChunkCtl + size_t(CTRAJ_MAX_TABLES) * kMaxSweepChunks * kCtlWords * sizeof(unsigned);
static_assert(CTRAJ_MAX_TABLES * kCtlWords * sizeof(unsigned) <= kSwChunkCtl, "sweep control layout");

unsigned* sweep_chunk_ctl(const ctraj_context* c, int t, size_t k) {
  return c->sweep_ctl.as<unsigned>(kSwChunkCtl + (size_t(t) * kMaxSweepChunks + k) * kCtlWords * sizeof(unsigned));
}

// Estimated largest RK4 step count of the sweep's molecules in the lens:
// exact in dz mode; in dt mode from the slowest vz expected (five standard
// deviations below the mean of drawn velocities, the smallest positive vz of
// host initial conditions).  0 when unknown.  It only shapes the chunk
// sequence: the last chunk has no step limit.
int64_t sweep_step_estimate(const ctraj_element& e, const ctraj_run_args* a) {
  const double L = e.p[7];
  double n = 0.0;
  if (e.step_mode != CTRAJ_STEP_DT) {
    n = std::fabs(std::rint(L / e.p[1]));
  } else {
    double vz = 0.0;
    if (a->ic_mode == CTRAJ_IC_DEVICE_DRAW) {
      const double mu = a->vdist.p[4], sg = std::fabs(a->vdist.p[5]);
      vz = std::max(mu - 5.0 * sg, 0.2 * mu);
    } else if (a->ic_mode == CTRAJ_IC_HOST) {
      vz = INFINITY;
      const double* v = a->ics + size_t(5) * size_t(a->n);
      for (int64_t i = 0; i < a->n; ++i)
        if (v[i] > 0.0 && v[i] < vz) vz = v[i];
    }
    if (vz > 0.0 && std::isfinite(vz)) n = L / (vz * e.p[2]);
  }
  if (!std::isfinite(n) || n <= 0.0) return 0;
  return int64_t(std::min(n, double(CTRAJ_MAX_LENS_STEPS))) + 1;
}

// Geometric chunk lengths (the context's tuning) until the estimate is
// covered, then one chunk without a step limit.
std::vector<int> sweep_chunks(const ctraj_context* c, int64_t est) {
  std::vector<int> v;
  int64_t done = 0, len = c->chunk;
  if (est == 0) est = c->chunk_max;
  while (done < est && int(v.size()) < kMaxSweepChunks - 1) {
    v.push_back(int(len));
    done += len;
    len = std::min<int64_t>(std::max<int64_t>(len + 1, len * c->chunk_growth / 100), c->chunk_max);
  }
  v.push_back(0x7fffffff);
  return v;
}

LensKernel sweep_lens_kernel(int force, bool staged) {
  using M = Mol32<false, false>;
  if (force == kForceStark2Lin)
    return staged ? k_lens_chunk<M, false, kForceStark2Lin, false, true, true>
                  : k_lens_chunk<M, false, kForceStark2Lin, false, false, true>;
  if (staged)
    return force == kForceStark1 ? k_lens_chunk<M, false, kForceStark1, false, true, true>
                                 : k_lens_chunk<M, false, kForceStark2, false, true, true>;
  return force == kForceStark1 ? k_lens_chunk<M, false, kForceStark1, false, false, true>
                               : k_lens_chunk<M, false, kForceStark2, false, false, true>;
}

struct SweepLaunch {
  int n_tab = 0;
  int lens = 0;
  Queue qa[CTRAJ_MAX_TABLES], qb[CTRAJ_MAX_TABLES];  // entrance / ping-pong storage per table
  LensArgs la[CTRAJ_MAX_TABLES];
  std::vector<int> chunks;
  unsigned long long* result = nullptr;  // device: per-configuration counts | totals | stats
  size_t result_bytes = 0;
  bool persistent = false;               // one k_sweep_persist launch instead of the chunks
  int force = kForceStark2;              // the lens's force law; kForceStark2Lin when every table
                                         // passes the linear form's test at its largest voltage
  unsigned* order[CTRAJ_MAX_TABLES] = {};  // persistent: bucket counts then entrant order, per table
};

// The persistent sweep lens kernel of a force law; staged when every table fits.
using SweepPersistKernel = void (*)(const Plan, const RunDev, const int, const SweepQueues, const int,
                                    const SweepTabs, const LensArgs, const int);
SweepPersistKernel sweep_persist_kernel(int force, bool staged) {
  if (force == kForceStark2Lin)
    return staged ? k_sweep_persist<kForceStark2Lin, true> : k_sweep_persist<kForceStark2Lin, false>;
  if (staged)
    return force == kForceStark1 ? k_sweep_persist<kForceStark1, true> : k_sweep_persist<kForceStark2, true>;
  return force == kForceStark1 ? k_sweep_persist<kForceStark1, false> : k_sweep_persist<kForceStark2, false>;
}

bool sweep_staged(const SweepLaunch& W) {
  for (int t = 0; t < W.n_tab; ++t)
    if (W.la[t].n_smem == 0) return false;
  return true;
}

size_t sweep_persist_smem(const SweepLaunch& W) {
  int max_int = 0;
  for (int t = 0; t < W.n_tab; ++t) max_int = std::max(max_int, W.la[t].n_int);
  return (sweep_staged(W) ? size_t(max_int) * sizeof(float4) : 0) + kPersistThreads * sizeof(SwapSlot);
}

// The whole sweep on c->stream (forking to one side stream per table).  Every
// call ends with the result copied to c->sweep_host; the caller synchronizes.
// While capturing, the timing events become event-record nodes of the graph.
int sweep_enqueue(ctraj_context* c, const Plan& P, const RunDev& R, const SweepLaunch& W, bool capturing) {
  cudaStream_t s = c->stream;
  int launches = 0;
  auto record = [&](cudaEvent_t ev) {
    return capturing ? cudaEventRecordWithFlags(ev, s, cudaEventRecordExternal) : cudaEventRecord(ev, s);
  };
  CT_CUDA(cudaMemsetAsync(c->sweep_ctl.p, 0, kSwCtlBytes, s));
  CT_CUDA(cudaMemsetAsync(W.result, 0, W.result_bytes, s));
  if (c->timing) CT_CUDA(record(c->ev[0]));
  if (R.n > 0) {
    auto kf = k_sweep_front<Mol32<false, false>>;
    const int ft = c->front_threads;
    const int bps = blocks_per_sm(kf, ft, 0);
    const int64_t want = (R.n + ft - 1) / ft;
    const int grid = int(std::min<int64_t>(want, int64_t(bps) * c->sm_count * c->front_waves));
    SweepQueues Qs{};
    for (int t = 0; t < W.n_tab; ++t) Qs.q[t] = W.qa[t];
    kf<<<grid, ft, 0, s>>>(P, R, Qs, W.n_tab);
    CT_CUDA(cudaGetLastError());
    ++launches;
  }
  if (c->timing) CT_CUDA(record(c->ev[1]));
  if (W.persistent && R.n > 0) {
    SweepQueues Qs{};
    SweepTabs T{};
    for (int t = 0; t < W.n_tab; ++t) {
      Qs.q[t] = W.qa[t];
      unsigned* hist = W.order[t];
      CT_CUDA(cudaMemsetAsync(hist, 0, kOrderBuckets * sizeof(unsigned), s));
      k_order_count<<<c->sm_count, kOrderThreads, 0, s>>>(P, W.lens, W.qa[t], hist);
      k_order_scan<<<1, kOrderBuckets, 0, s>>>(hist);
      k_order_place<<<c->sm_count, kOrderThreads, 0, s>>>(P, W.lens, W.qa[t], hist, hist + kOrderBuckets);
      CT_CUDA(cudaGetLastError());
      launches += 3;
      T.q[t] = W.la[t].q;
      T.order[t] = hist + kOrderBuckets;
      T.s0[t] = W.la[t].s0;
      T.n_int[t] = W.la[t].n_int;
    }
    sweep_persist_kernel(W.force, sweep_staged(W))<<<c->sm_count, kPersistThreads,
                                                                  sweep_persist_smem(W), s>>>(
        P, R, W.lens, Qs, W.n_tab, T, W.la[0], c->lens_interval);
    CT_CUDA(cudaGetLastError());
    ++launches;
    if (c->timing) CT_CUDA(record(c->ev[3]));
    CT_CUDA(cudaMemcpyAsync(c->sweep_host, W.result, W.result_bytes, cudaMemcpyDeviceToHost, s));
    c->sweep_launches = launches;
    return CTRAJ_OK;
  }
  CT_CUDA(cudaEventRecord(c->fork, s));
  for (int t = 0; t < W.n_tab && R.n > 0; ++t) {
    cudaStream_t st = c->side[t];
    CT_CUDA(cudaStreamWaitEvent(st, c->fork, 0));
    const bool staged = W.la[t].n_smem > 0;
    const size_t smem = staged ? size_t(W.la[t].n_int) * sizeof(float4) : 0;
    LensKernel kl = sweep_lens_kernel(W.force, staged);
    const int grid = blocks_per_sm(kl, kLensThreads, smem) * c->sm_count;
    Queue in = W.qa[t];
    for (size_t k = 0; k < W.chunks.size(); ++k) {
      Queue out = (k & 1) ? W.qa[t] : W.qb[t];
      out.count = sweep_chunk_ctl(c, t, k);
      out.max_steps = out.count + 1;
      out.head = out.count + 2;
      // nothing follows the sweep's only lens: the next-lens queue is never written
      kl<<<grid, kLensThreads, smem, st>>>(P, R, W.lens, in, out, out, W.chunks[k], W.la[t]);
      CT_CUDA(cudaGetLastError());
      ++launches;
      in = out;
    }
    CT_CUDA(cudaEventRecord(c->join[t], st));
    CT_CUDA(cudaStreamWaitEvent(s, c->join[t], 0));
  }
  if (c->timing) CT_CUDA(record(c->ev[3]));
  CT_CUDA(cudaMemcpyAsync(c->sweep_host, W.result, W.result_bytes, cudaMemcpyDeviceToHost, s));
  c->sweep_launches = launches;
  return CTRAJ_OK;
}

int validate_sweep(const ctraj_context* c, const ctraj_sweep* sw, const ctraj_run_args* a,
                   const int64_t* counts, int* lens) {
  if (!sw || !counts) return fail(CTRAJ_EINVAL, "NULL argument");
  if (a->precision != 32) return fail(CTRAJ_EINVAL, "sweeps run in precision 32 only");
  if (a->out_mode != CTRAJ_OUT_NONE) return fail(CTRAJ_EINVAL, "sweeps take out_mode CTRAJ_OUT_NONE");
  if (sw->n_configs < 1 || sw->n_configs > CTRAJ_MAX_SWEEP_CONFIGS)
    return fail(CTRAJ_EINVAL, "n_configs %d out of range [1, %d]", sw->n_configs, CTRAJ_MAX_SWEEP_CONFIGS);
  if (!sw->n_molecules || !sw->alpha || !sw->table) return fail(CTRAJ_EINVAL, "sweep arrays are NULL");
  int n_lens = 0;
  for (size_t i = 0; i < c->elements.size(); ++i)
    if (c->elements[i].type == CTRAJ_ELECTROSTATIC_LENS) {
      ++n_lens;
      *lens = int(i);
    }
  if (n_lens != 1) return fail(CTRAJ_EINVAL, "a sweep beamline needs exactly one lens (it has %d)", n_lens);
  const ctraj_element& e = c->elements[*lens];
  if (e.field_order != 1 && e.field_order != 2)
    return fail(CTRAJ_EINVAL, "the sweep lens needs a Stark force law (field_order 1 or 2)");
  int64_t total = 0;
  for (int k = 0; k < sw->n_configs; ++k) {
    if (sw->n_molecules[k] < 0) return fail(CTRAJ_EINVAL, "configuration %d: negative n_molecules", k);
    total += sw->n_molecules[k];
    if (total > a->n) break;
    const int id = sw->table[k];
    if (id < 0 || id >= CTRAJ_MAX_TABLES || !c->tables[id].n)
      return fail(CTRAJ_ESTATE, "configuration %d uses force table %d, which is not set", k, id);
    if (c->tables[id].kind != CTRAJ_TABLE_STARK_SPLINE)
      return fail(CTRAJ_EINVAL, "configuration %d: table %d is not a Stark spline table", k, id);
    if (!std::isfinite(sw->alpha[k])) return fail(CTRAJ_EINVAL, "configuration %d: alpha is not finite", k);
  }
  if (total != a->n)
    return fail(CTRAJ_EINVAL, "the configurations' n_molecules do not add up to args->n = %lld", (long long)a->n);
  return CTRAJ_OK;
}

}  // namespace
}  // namespace ctraj

extern "C" int ctraj_run_sweep(ctraj_context* c, const ctraj_sweep* sw, const ctraj_run_args* a,
                               int64_t* counts, ctraj_run_stats* stats) {
  if (!c) return fail(CTRAJ_EINVAL, "ctx is NULL");
  int st = validate_run(c, a);
  if (st) return st;
  int lens = 0;
  if ((st = validate_sweep(c, sw, a, counts, &lens))) return st;
  Plan P;
  RunDev R;
  if ((st = prepare(c, a, P, R))) return st;
  const ctraj_element& e = c->elements[lens];
  const int n_cfg = sw->n_configs;
  const int nl = c->n_labels;

  // dense table index per configuration, molecules per table
  SweepLaunch W;
  W.lens = lens;
  int dense_of[CTRAJ_MAX_TABLES];
  std::fill(dense_of, dense_of + CTRAJ_MAX_TABLES, -1);
  int tab_id[CTRAJ_MAX_TABLES];
  int64_t tab_n[CTRAJ_MAX_TABLES] = {};
  for (int k = 0; k < n_cfg; ++k) {
    const int id = sw->table[k];
    if (dense_of[id] < 0) {
      dense_of[id] = W.n_tab;
      tab_id[W.n_tab++] = id;
    }
    tab_n[dense_of[id]] += sw->n_molecules[k];
  }
  // the table form: linear pieces when every table passes the test with the
  // largest field coefficient any of its configurations uses
  W.force = e.field_order == 1 ? kForceStark1 : kForceStark2;
  if (e.field_order == 2) {
    double alpha_max[CTRAJ_MAX_TABLES];
    std::fill(alpha_max, alpha_max + CTRAJ_MAX_TABLES, 0.0);
    bool lin = true;
    for (int k = 0; k < n_cfg; ++k) {
      const int d = dense_of[sw->table[k]];
      if (!(sw->alpha[k] >= 0.0)) lin = false;
      alpha_max[d] = std::max(alpha_max[d], sw->alpha[k]);
    }
    for (int t = 0; t < W.n_tab && lin; ++t) {
      const HostTable& ht = c->tables[tab_id[t]];
      ctraj_element ex = e;
      ex.p[6] = alpha_max[t];
      lin = stark_linear(ht.kind, ht.n, ht.knots.data(), ht.coef.data(), ex);
    }
    if (lin) W.force = kForceStark2Lin;
  }
  const bool lin = W.force == kForceStark2Lin;
  const double piece_scale = lin ? double(kLinearPieces) : 1.0;  // table coordinate units per knot interval

  // buffers (grow-only); any reallocation invalidates a captured graph
  bool moved = false;
  auto ens = [&](DevBuf& b, size_t want) {
    if (want > b.bytes) moved = true;
    return b.ensure(want);
  };
  size_t tab_off[CTRAJ_MAX_TABLES], tab_elems = 0;
  for (int t = 0; t < W.n_tab; ++t) {
    tab_off[t] = tab_elems;
    tab_elems += size_t(c->tables[tab_id[t]].n - 1) * (lin ? 2 : 1);
  }
  const size_t words = size_t(n_cfg) * (nl + 1);
  const size_t cfg_bytes = align256(size_t(n_cfg + 1) * 8) + 3 * align256(size_t(n_cfg) * 4);
  W.result_bytes = (words + CTRAJ_MAX_LABELS + 1 + kStatCount) * 8;
  if ((st = ens(c->sweep_tables, tab_elems * sizeof(float4)))) return st;
  if ((st = ens(c->sweep_cfg, cfg_bytes + W.result_bytes))) return st;
  if ((st = ens(c->sweep_ctl, kSwCtlBytes))) return st;
  W.persistent = c->lens_mode == CTRAJ_LENS_PERSISTENT;
  if (W.persistent) {
    size_t words_o = 0;
    for (int t = 0; t < W.n_tab; ++t) words_o += kOrderBuckets + size_t(std::max<int64_t>(tab_n[t], 1));
    if ((st = ens(c->sweep_order, words_o * sizeof(unsigned)))) return st;
    size_t off = 0;
    for (int t = 0; t < W.n_tab; ++t) {
      W.order[t] = c->sweep_order.as<unsigned>() + off;
      off += kOrderBuckets + size_t(std::max<int64_t>(tab_n[t], 1));
    }
  }
  for (int t = 0; t < W.n_tab; ++t) {
    const size_t cap = size_t(std::max<int64_t>(tab_n[t], 1));
    if ((st = ens(c->sweep_queue[2 * t], queue_bytes(cap, 32, true)))) return st;
    if ((st = ens(c->sweep_queue[2 * t + 1], queue_bytes(cap, 32, true)))) return st;
    layout_queue(&c->sweep_queue[2 * t], cap, 32, c->sweep_ctl.as<unsigned>(size_t(t) * kCtlWords * 4), &W.qa[t], true);
    layout_queue(&c->sweep_queue[2 * t + 1], cap, 32, nullptr, &W.qb[t], true);
  }
  const size_t host_words = W.result_bytes / 8;
  if (host_words > c->sweep_host_words) {
    if (c->sweep_host) cudaFreeHost(c->sweep_host);
    c->sweep_host = nullptr;
    c->sweep_host_words = 0;
    CT_CUDA(cudaMallocHost(&c->sweep_host, host_words * 8));
    c->sweep_host_words = host_words;
    moved = true;
  }
  for (int t = 0; t < W.n_tab; ++t) {
    if (!c->side[t]) CT_CUDA(cudaStreamCreateWithFlags(&c->side[t], cudaStreamNonBlocking));
    if (!c->join[t]) CT_CUDA(cudaEventCreateWithFlags(&c->join[t], cudaEventDisableTiming));
  }
  if (!c->fork) CT_CUDA(cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming));
  if (moved) ++c->generation;

  // device views
  char* cb = c->sweep_cfg.as<char>();
  int64_t* d_start = reinterpret_cast<int64_t*>(cb);
  float* d_beta = reinterpret_cast<float*>(cb + align256(size_t(n_cfg + 1) * 8));
  float* d_kappa = reinterpret_cast<float*>(reinterpret_cast<char*>(d_beta) + align256(size_t(n_cfg) * 4));
  int32_t* d_table = reinterpret_cast<int32_t*>(reinterpret_cast<char*>(d_kappa) + align256(size_t(n_cfg) * 4));
  W.result = reinterpret_cast<unsigned long long*>(cb + cfg_bytes);
  R.n_cfg = n_cfg;
  R.cfg_start = d_start;
  R.cfg_beta = d_beta;
  R.cfg_kappa = d_kappa;
  R.cfg_table = d_table;
  R.cfg_counts = W.result;
  R.counts = W.result + words;
  R.stats = W.result + words + CTRAJ_MAX_LABELS + 1;

  const double mass = e.p[5];
  for (int t = 0; t < W.n_tab; ++t) {
    const HostTable& ht = c->tables[tab_id[t]];
    const double h = (ht.knots[ht.n - 1] - ht.knots[0]) / double(ht.n - 1);
    LensArgs& L = W.la[t];
    L = lens_args(P, lens, true);
    L.q = c->sweep_tables.as<float4>(tab_off[t] * sizeof(float4));
    L.beta = 0.f;  // per configuration
    L.s0 = float(piece_scale * ht.knots[0] / h);
    L.r_max = INFINITY;
    L.n_int = (ht.n - 1) * (lin ? 2 : 1);  // float4 entries
    L.n_smem = L.n_int <= (lin ? kMaxStagedLinear : kMaxStagedIntervals) ? L.n_int : 0;
  }
  W.chunks = sweep_chunks(c, sweep_step_estimate(e, a));

  // what a captured graph depends on
  std::vector<char> key;
  auto put = [&](const void* p, size_t n) {
    key.insert(key.end(), static_cast<const char*>(p), static_cast<const char*>(p) + n);
  };
  const int timing = a->timing != 0;
  put(&c->generation, sizeof c->generation);
  put(&c->stream, sizeof c->stream);
  put(&timing, sizeof timing);
  put(&P, sizeof P);
  put(&R, sizeof R);
  put(sw->n_molecules, size_t(n_cfg) * 8);
  put(sw->alpha, size_t(n_cfg) * 8);
  put(sw->table, size_t(n_cfg) * 4);
  put(W.chunks.data(), W.chunks.size() * sizeof(int));
  put(&c->lens_mode, sizeof c->lens_mode);
  put(&c->lens_interval, sizeof c->lens_interval);
  put(&c->front_threads, sizeof c->front_threads);
  put(&W.force, sizeof W.force);
  const bool same = key == c->sweep_key;
  cudaStream_t s = c->stream;
  if (!same) {
    // unscaled tables: W'(E) = q.x + q.y u + q.z u^2 in interval j, u = (E - E_j) / h,
    // or its quarter-interval linear pieces
    std::vector<float4> host(tab_elems);
    for (int t = 0; t < W.n_tab; ++t) {
      const HostTable& ht = c->tables[tab_id[t]];
      const double h = (ht.knots[ht.n - 1] - ht.knots[0]) / double(ht.n - 1);
      for (int j = 0; j < ht.n - 1; ++j) {
        const double* cj = &ht.coef[size_t(j) * 4];
        const double qa = cj[2], qb = 2.0 * cj[1] * h, qc = 3.0 * cj[0] * h * h;
        if (lin) {
          host[tab_off[t] + 2 * j] = stark_pieces(qa, qb, qc, 0);
          host[tab_off[t] + 2 * j + 1] = stark_pieces(qa, qb, qc, 1);
        } else {
          host[tab_off[t] + j] = make_float4(float(qa), float(qb), float(qc), 0.f);
        }
      }
    }
    // per configuration: first molecule, beta = alpha / h, kappa = -(n alpha / m) (n = field order)
    std::vector<char> hc(cfg_bytes);
    int64_t* h_start = reinterpret_cast<int64_t*>(hc.data());
    float* h_beta = reinterpret_cast<float*>(hc.data() + (reinterpret_cast<char*>(d_beta) - cb));
    float* h_kappa = reinterpret_cast<float*>(hc.data() + (reinterpret_cast<char*>(d_kappa) - cb));
    int32_t* h_table = reinterpret_cast<int32_t*>(hc.data() + (reinterpret_cast<char*>(d_table) - cb));
    h_start[0] = 0;
    for (int k = 0; k < n_cfg; ++k) {
      h_start[k + 1] = h_start[k] + sw->n_molecules[k];
      const int id = sw->table[k];
      const HostTable& ht = c->tables[id];
      const double h = (ht.knots[ht.n - 1] - ht.knots[0]) / double(ht.n - 1);
      const double alpha = sw->alpha[k];
      h_beta[k] = float(piece_scale * alpha / h);
      h_kappa[k] = float(-(e.field_order == 1 ? alpha / mass : 2.0 * alpha / mass));
      h_table[k] = dense_of[id];
    }
    if (tab_elems)
      CT_CUDA(cudaMemcpyAsync(c->sweep_tables.p, host.data(), tab_elems * sizeof(float4), cudaMemcpyHostToDevice, s));
    CT_CUDA(cudaMemcpyAsync(cb, hc.data(), cfg_bytes, cudaMemcpyHostToDevice, s));
    CT_CUDA(cudaStreamSynchronize(s));  // the host staging vectors go out of scope
    if (c->sweep_exec) {
      cudaGraphExecDestroy(c->sweep_exec);
      c->sweep_exec = nullptr;
    }
    c->sweep_key.swap(key);
  }
  for (int t = 0; t < W.n_tab; ++t) {
    const bool staged = W.la[t].n_smem > 0;
    const size_t smem = staged ? size_t(W.la[t].n_int) * sizeof(float4) : 0;
    CT_CUDA(cudaFuncSetAttribute(sweep_lens_kernel(W.force, staged),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  }
  if (W.persistent)
    CT_CUDA(cudaFuncSetAttribute(sweep_persist_kernel(W.force, sweep_staged(W)),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(sweep_persist_smem(W))));
  c->timing = timing;
  if (sw->use_graph) {
    if (!c->sweep_exec) {
      CT_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      const int est = sweep_enqueue(c, P, R, W, true);
      cudaGraph_t g = nullptr;
      const cudaError_t ec = cudaStreamEndCapture(s, &g);
      if (est) {
        if (g) cudaGraphDestroy(g);
        return est;
      }
      if (ec != cudaSuccess) return fail(CTRAJ_ECUDA, "sweep graph capture: %s", cudaGetErrorString(ec));
      const cudaError_t ei = cudaGraphInstantiate(&c->sweep_exec, g, 0);
      cudaGraphDestroy(g);
      if (ei != cudaSuccess) {
        c->sweep_exec = nullptr;
        return fail(CTRAJ_ECUDA, "sweep graph instantiation: %s", cudaGetErrorString(ei));
      }
    }
    CT_CUDA(cudaGraphLaunch(c->sweep_exec, s));
  } else {
    if ((st = sweep_enqueue(c, P, R, W, false))) return st;
  }
  CT_CUDA(cudaStreamSynchronize(s));
  const unsigned long long* hr = c->sweep_host;
  for (size_t k = 0; k < words; ++k) counts[k] = int64_t(hr[k]);
  for (int k = 0; k <= nl; ++k) a->counts[k] = int64_t(hr[words + k]);
  const unsigned long long* hs = hr + words + CTRAJ_MAX_LABELS + 1;
  if (stats) {
    std::memset(stats, 0, sizeof *stats);
    stats->molecules = a->n;
    stats->molecule_steps = int64_t(hs[kStatSteps]);
    stats->lens_steps = int64_t(hs[kStatLensSteps]);
    stats->edge_band = -1;
    stats->table_range = int64_t(hs[kStatTableRange]);
    stats->bad_steps = int64_t(hs[kStatBadSteps]);
    stats->kernels = c->sweep_launches;
    if (timing) {
      stats->timed = 1;
      CT_CUDA(cudaEventElapsedTime(&stats->front_ms, c->ev[0], c->ev[1]));
      CT_CUDA(cudaEventElapsedTime(&stats->lens_ms, c->ev[1], c->ev[3]));
    }
  }
  if (hs[kStatBadSteps])
    return fail(CTRAJ_ESTEPS, "%llu molecules have a non-finite or oversize lens step count rint(L/dz)",
                hs[kStatBadSteps]);
  return CTRAJ_OK;
}

// ============================================================================
// Soft transmission and its discrete adjoint (ctraj_soft_transmission)
// ============================================================================
namespace ctraj {
namespace {

int soft_plan(const ctraj_context* c, const ctraj_soft_args* a, const double* prm, SoftPlan& S, int* lens) {
  std::memset(&S, 0, sizeof S);
  const int n_el = int(c->elements.size());
  int li = -1;
  for (int i = 0; i < n_el; ++i)
    if (c->elements[i].type == CTRAJ_ELECTROSTATIC_LENS) {
      if (li >= 0) return fail(CTRAJ_EINVAL, "soft transmission: the beamline has more than one lens");
      li = i;
    }
  if (li < 0) return fail(CTRAJ_EINVAL, "soft transmission: the beamline has no lens");
  const ctraj_element& L = c->elements[li];
  const HostTable& t = c->tables[L.table];
  if (t.kind != CTRAJ_TABLE_STARK_SPLINE || L.field_order != 2)
    return fail(CTRAJ_EINVAL, "soft transmission needs a Stark spline lens with field order 2");
  if (a->aperture >= 0 && (a->aperture >= li || c->elements[a->aperture].type != CTRAJ_CIRCULAR_APERTURE))
    return fail(CTRAJ_EINVAL, "soft transmission: element %d is not a circular aperture in front of the lens",
                a->aperture);
  int np = 0;
  for (int i = 0; i < li; ++i) {
    const ctraj_element& e = c->elements[i];
    if (e.type != CTRAJ_CIRCULAR_APERTURE)
      return fail(CTRAJ_EINVAL, "soft transmission: element %d in front of the lens is not a circular aperture", i);
    const double r = i == a->aperture ? prm[CTRAJ_SOFT_APERTURE_R] : e.p[0] * 0.5;
    for (int k = 0; k < 2; ++k) {
      S.z[np] = k ? e.z1 : e.z0;
      S.radius[np] = std::isinf(r) ? INFINITY : r;
      S.param[np] = i == a->aperture;
      ++np;
    }
  }
  for (int i = li + 1; i < n_el; ++i) {
    const ctraj_element& e = c->elements[i];
    if (e.type != CTRAJ_CIRCULAR_APERTURE || !std::isinf(e.p[0]))
      return fail(CTRAJ_EINVAL, "soft transmission: element %d behind the lens must be a plane of infinite diameter", i);
  }
  S.z[np] = prm[CTRAJ_SOFT_LENS_Z0];  // the lens entrance
  S.radius[np] = INFINITY;
  ++np;
  S.n_planes = np;
  S.n = a->n;
  S.seed = a->seed;
  S.key = philox_key(a->seed);
  S.offset = a->offset;
  S.ic_mode = a->ic_mode;
  S.z_ic = a->xdist.p[2];
  S.sx = a->xdist.p[0];
  S.sy = a->xdist.p[1];
  S.mu_vx = a->vdist.p[0];
  S.mu_vy = a->vdist.p[2];
  S.mu_vz = a->vdist.p[4];
  S.s_vz = a->vdist.p[5];
  S.s_vx = prm[CTRAJ_SOFT_SIGMA_VX];
  S.s_vy = prm[CTRAJ_SOFT_SIGMA_VY];
  S.lens = L;
  S.lens.z0 = prm[CTRAJ_SOFT_LENS_Z0];
  S.lens.z1 = S.lens.z0 + L.p[7];
  const double V = prm[CTRAJ_SOFT_V], R = L.p[4], mass = L.p[5];
  const double h = (t.knots[t.n - 1] - t.knots[0]) / double(t.n - 1);
  const double alpha = 3.0 * V / (R * R * R);
  S.V = V;
  S.beta = alpha / h;
  S.s0 = t.knots[0] / h;
  S.kappa = -2.0 * alpha / mass;
  S.kappa1 = -2.0 * 3.0 / (R * R * R) / mass;
  S.bore = prm[CTRAJ_SOFT_BORE_R];
  S.inv_w = 1.0 / a->width;
  S.g = a->g;
  S.log_floor = a->log_floor;
  S.n_int = t.n - 1;
  S.checkpoint = a->checkpoint;
  *lens = li;
  return CTRAJ_OK;
}

template <class T>
int soft_run(ctraj_context* c, const ctraj_soft_args* a, SoftPlan& S, int li, ctraj_soft_result* out) {
  cudaStream_t s = c->stream;
  const HostTable& t = c->tables[c->elements[li].table];
  const double h = (t.knots[t.n - 1] - t.knots[0]) / double(t.n - 1);
  // table f W'(E) = q0 + q1 u + q2 u^2 on each interval, in T, with a power of
  // two f that brings the largest coefficient near 1 (W' is ~1e-29 J m/V and
  // kappa beta ~1e40 would overflow float); kappa and kappa1 carry 1/f
  double qmax = 0.0;
  for (int j = 0; j < t.n - 1; ++j) {
    const double* cj = &t.coef[size_t(j) * 4];
    qmax = std::max({qmax, std::fabs(cj[2]), std::fabs(2.0 * cj[1] * h), std::fabs(3.0 * cj[0] * h * h)});
  }
  const double f = qmax > 0.0 && std::isfinite(qmax) ? std::ldexp(1.0, -std::ilogb(qmax)) : 1.0;
  S.kappa /= f;
  S.kappa1 /= f;
  std::vector<Coef4<T>> host(t.n - 1);
  for (int j = 0; j < t.n - 1; ++j) {
    const double* cj = &t.coef[size_t(j) * 4];
    host[j] = Coef4<T>{T(f * cj[2]), T(f * (2.0 * cj[1] * h)), T(f * (3.0 * cj[0] * h * h)), T(0)};
  }
  const size_t tb = host.size() * sizeof(Coef4<T>);
  if (tb > 200 * 1024) return fail(CTRAJ_EINVAL, "soft transmission: the lens table (%d knots) is too large", t.n);
  int st;
  const int64_t chunk = std::min<int64_t>(std::max<int64_t>(a->n, 1), kSoftChunk);
  if ((st = c->soft_table.ensure(tb))) return st;
  if ((st = c->soft_queue.ensure(size_t(chunk) * 4 * 3))) return st;
  if ((st = c->soft_ctl.ensure(kSoftCtlBytes))) return st;
  if ((st = c->soft_contrib.ensure(size_t(chunk) * kSoftAcc * 8))) return st;
  CT_CUDA(cudaMemcpyAsync(c->soft_table.p, host.data(), tb, cudaMemcpyHostToDevice, s));
  if (a->ic_mode == CTRAJ_IC_HOST && a->n > 0) {
    const size_t b = size_t(a->n) * 5 * 8;
    if ((st = c->ics.ensure(b))) return st;
    CT_CUDA(cudaMemcpyAsync(c->ics.p, a->normals, b, cudaMemcpyHostToDevice, s));
    S.normals = c->ics.as<double>();
  }
  SoftQueue Q{c->soft_queue.as<int32_t>(), c->soft_ctl.as<unsigned>(0), c->soft_ctl.as<unsigned>(4),
              c->soft_queue.as<int32_t>(size_t(chunk) * 4), c->soft_queue.as<int32_t>(size_t(chunk) * 8),
              c->soft_ctl.as<unsigned>(8)};
  unsigned long long* stats = c->soft_ctl.as<unsigned long long>(256);
  double* partial = c->soft_ctl.as<double>(256 + 8 * kSoftStatCount);
  double* contrib = c->soft_contrib.as<double>();
  CT_CUDA(cudaMemsetAsync(stats, 0, 8 * kSoftStatCount, s));
  auto kl = a->want_grad ? k_soft_lens<T, true> : k_soft_lens<T, false>;
  CT_CUDA(cudaFuncSetAttribute(kl, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tb)));
  std::memset(out, 0, sizeof *out);
  double sum[kSoftAcc] = {};
  int launches = 0;
  float front_ms = 0.f, lens_ms = 0.f;
  // molecules in chunks of at most kSoftChunk: per chunk the front, the lens
  // pass and the fixed-order column sums, added on the host in chunk order
  for (int64_t first = 0; first < a->n; first += chunk) {
    S.first = first;
    S.count = std::min<int64_t>(chunk, a->n - first);
    CT_CUDA(cudaMemsetAsync(c->soft_ctl.p, 0, 256, s));
    CT_CUDA(cudaMemsetAsync(contrib, 0, size_t(S.count) * kSoftAcc * 8, s));
    if (a->timing) CT_CUDA(cudaEventRecord(c->ev[0], s));
    auto kf = k_soft_front<T>;
    const int bps = blocks_per_sm(kf, kThreads, 0);
    const int64_t want = (S.count + kThreads - 1) / kThreads;
    int grid = int(std::min<int64_t>(want, int64_t(bps) * c->sm_count * c->front_waves));
    kf<<<grid, kThreads, 0, s>>>(S, Q, stats);
    CT_CUDA(cudaGetLastError());
    ++launches;
    if (a->timing) CT_CUDA(cudaEventRecord(c->ev[1], s));
    CT_CUDA(cudaMemcpyAsync(c->host_max, Q.count, 2 * sizeof(unsigned), cudaMemcpyDeviceToHost, s));
    CT_CUDA(cudaStreamSynchronize(s));
    const unsigned count = c->host_max[0], max_steps = c->host_max[1];
    out->lens_molecules += int64_t(count);
    if (count > 0) {
      const size_t cap = count;
      const size_t n_seg = (size_t(max_steps) + S.checkpoint - 1) / S.checkpoint + 1;
      const int max_seg = int(n_seg - 1);
      if (a->want_grad) {
        if ((st = c->soft_ckpt.ensure(n_seg * 8 * cap * sizeof(T), 25))) return st;
        if ((st = c->soft_seg.ensure(size_t(kSoftSegFields) * cap * size_t(max_seg) * sizeof(T), 25))) return st;
      }
      grid = int((cap + kSoftThreads - 1) / kSoftThreads);
      kl<<<grid, kSoftThreads, tb, s>>>(S, Q, c->soft_table.as<Coef4<T>>(), c->soft_ckpt.as<T>(), cap, contrib,
                                         stats);
      CT_CUDA(cudaGetLastError());
      ++launches;
      if (a->want_grad && max_seg > 0) {
        // backward: every (survivor, segment) in parallel, then per survivor
        // the composition and the ballistic part; both read the survivor
        // count on the device
        auto ks = k_soft_seg<T>;
        CT_CUDA(cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tb)));
        const int gs = blocks_per_sm(ks, kSoftThreads, tb) * c->sm_count * 4;
        ks<<<gs, kSoftThreads, tb, s>>>(S, Q, c->soft_table.as<Coef4<T>>(), c->soft_ckpt.as<T>(), cap,
                                        c->soft_seg.as<T>(), max_seg, cap);
        CT_CUDA(cudaGetLastError());
        k_soft_compose<T><<<grid, kSoftThreads, 0, s>>>(S, Q, c->soft_seg.as<T>(), max_seg, cap, contrib);
        CT_CUDA(cudaGetLastError());
        launches += 2;
      }
    }
    k_soft_reduce<<<dim3(kSoftReduceBlocks, kSoftAcc), 256, 0, s>>>(contrib, S.count, partial);
    CT_CUDA(cudaGetLastError());
    ++launches;
    if (a->timing) CT_CUDA(cudaEventRecord(c->ev[3], s));
    double hp[kSoftAcc * kSoftReduceBlocks];
    CT_CUDA(cudaMemcpyAsync(hp, partial, sizeof hp, cudaMemcpyDeviceToHost, s));
    CT_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < kSoftAcc; ++k)
      for (int b = 0; b < kSoftReduceBlocks; ++b) sum[k] += hp[k * kSoftReduceBlocks + b];
    if (a->timing) {
      float f0 = 0.f, f1 = 0.f;
      CT_CUDA(cudaEventElapsedTime(&f0, c->ev[0], c->ev[1]));
      CT_CUDA(cudaEventElapsedTime(&f1, c->ev[1], c->ev[3]));
      front_ms += f0;
      lens_ms += f1;
    }
  }
  unsigned long long hs[kSoftStatCount];
  CT_CUDA(cudaMemcpyAsync(hs, stats, sizeof hs, cudaMemcpyDeviceToHost, s));
  CT_CUDA(cudaStreamSynchronize(s));
  const double inv_n = a->n > 0 ? 1.0 / double(a->n) : 0.0;
  out->loss = sum[0] * inv_n;
  for (int k = 0; k < kSoftParams; ++k) out->grad[k] = a->want_grad ? sum[1 + k] * inv_n : 0.0;
  out->lens_steps = int64_t(hs[kSoftStatSteps]);
  out->dropped = int64_t(hs[kSoftStatDropped]);
  out->bad_steps = int64_t(hs[kSoftStatBad]);
  out->kernels = launches;
  if (a->timing) {
    out->timed = 1;
    out->front_ms = front_ms;
    out->lens_ms = lens_ms;
  }
  return CTRAJ_OK;
}

}  // namespace
}  // namespace ctraj

extern "C" int ctraj_soft_transmission(ctraj_context* c, const ctraj_soft_args* a, const double* params,
                                       ctraj_soft_result* out) {
  if (!c || !a || !params || !out) return fail(CTRAJ_EINVAL, "NULL argument");
  if (!c->have_beamline) return fail(CTRAJ_ESTATE, "ctraj_set_beamline was not called");
  if (a->n < 0 || a->n > int64_t(0x7fffffff)) return fail(CTRAJ_EINVAL, "n = %lld out of range", (long long)a->n);
  if (a->precision != 32 && a->precision != 64) return fail(CTRAJ_EINVAL, "precision must be 32 or 64");
  if (a->ic_mode != CTRAJ_IC_DEVICE_DRAW && a->ic_mode != CTRAJ_IC_HOST)
    return fail(CTRAJ_EINVAL, "soft transmission: ic_mode must be CTRAJ_IC_DEVICE_DRAW or CTRAJ_IC_HOST");
  if (a->ic_mode == CTRAJ_IC_HOST && a->n > 0 && !a->normals) return fail(CTRAJ_EINVAL, "normals is NULL");
  if (a->xdist.kind != CTRAJ_DIST_GAUSSIAN_POSITION || a->vdist.kind != CTRAJ_DIST_GAUSSIAN_VELOCITY)
    return fail(CTRAJ_EINVAL, "soft transmission needs Gaussian position and velocity distributions");
  if (!(a->width > 0.0) || !std::isfinite(a->width)) return fail(CTRAJ_EINVAL, "width must be positive");
  if (a->checkpoint < 1 || a->checkpoint > kSoftTape)
    return fail(CTRAJ_EINVAL, "checkpoint must be in [1, %d]", kSoftTape);
  if (!std::isfinite(a->log_floor) || a->log_floor >= 0.0) return fail(CTRAJ_EINVAL, "log_floor must be negative");
  for (int k = 0; k < CTRAJ_SOFT_NPARAMS; ++k)
    if (!std::isfinite(params[k])) return fail(CTRAJ_EINVAL, "params[%d] is not finite", k);
  int st = check_beamline(c);
  if (st) return st;
  CT_CUDA(cudaSetDevice(c->device));
  SoftPlan S;
  int li = 0;
  if ((st = soft_plan(c, a, params, S, &li))) return st;
  return a->precision == 32 ? soft_run<float>(c, a, S, li, out) : soft_run<double>(c, a, S, li, out);
}

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
    int st = launch_front<Mol32<kOut, false>, kOut, kModePlain>(P, R, q[0], n, kThreads, sms, 4, s);
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
    int st = enqueue_persistent<kOut>(P, R, i, q[cur], q[nxt], order_buf, sms, 256, s, launches);
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
