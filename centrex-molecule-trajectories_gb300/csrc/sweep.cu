// libctraj.so: the batched sweep (ctraj_run_sweep, declared in include/ctraj.h):
// one front launch over every configuration's molecules, then per Stark table
// a persistent or chunked lens pass; optionally captured once as a CUDA graph.
#include "engine.h"
#include "kernels.cuh"

using namespace ctraj;

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
  DoneRec* done[CTRAJ_MAX_TABLES] = {};    // persistent: the molecules' end records, per table
  unsigned done_cap[CTRAJ_MAX_TABLES] = {};
  int outward = 0;                         // every configuration's force points away from the axis
  int threads = kPersistThreads;           // persistent: threads per CTA of k_sweep_persist
};

// The persistent sweep lens kernel of a force law; staged when every table
// fits.  Linear tables staged in shared memory run with `threads` (512, 768
// or 1024) per CTA, the others with 512.
using SweepPersistKernel = void (*)(const Plan, const RunDev, const int, const SweepQueues, const int,
                                    const SweepTabs, const LensArgs, const int, const int);
SweepPersistKernel sweep_persist_kernel(int force, bool staged, int threads) {
  if (force == kForceStark2Lin && staged) {
    if (threads == 768) return k_sweep_persist<kForceStark2Lin, true, 768>;
    if (threads == 1024) return k_sweep_persist<kForceStark2Lin, true, 1024>;
    return k_sweep_persist<kForceStark2Lin, true>;
  }
  if (force == kForceStark2Lin) return k_sweep_persist<kForceStark2Lin, false>;
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
  return (sweep_staged(W) ? size_t(max_int) * sizeof(float4) : 0) + size_t(W.threads) * sizeof(SwapSlot);
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
    const size_t fsmem = sweep_front_smem(ft);  // its size limit is set before any capture (below)
    const int bps = blocks_per_sm(kf, ft, fsmem);
    const int64_t want = (R.n + ft - 1) / ft;
    const int grid = int(std::min<int64_t>(want, int64_t(bps) * c->sm_count * c->front_waves));
    SweepQueues Qs{};
    for (int t = 0; t < W.n_tab; ++t) Qs.q[t] = W.qa[t];
    kf<<<grid, ft, fsmem, s>>>(P, R, Qs, W.n_tab);
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
      k_order_count<<<c->sm_count, kOrderThreads, 0, s>>>(P, W.lens, W.qa[t], hist, W.outward);
      k_order_scan<<<1, kOrderBuckets, 0, s>>>(hist);
      k_order_place<<<c->sm_count, kOrderThreads, 0, s>>>(P, W.lens, W.qa[t], hist, hist + kOrderBuckets,
                                                          W.outward);
      CT_CUDA(cudaGetLastError());
      launches += 3;
      T.q[t] = W.la[t].q;
      T.order[t] = hist + kOrderBuckets;
      T.s0[t] = W.la[t].s0;
      T.n_int[t] = W.la[t].n_int;
      T.done[t] = W.done[t];
      T.done_cap[t] = W.done_cap[t];
    }
    sweep_persist_kernel(W.force, sweep_staged(W), W.threads)<<<c->sm_count, W.threads,
                                                                             sweep_persist_smem(W), s>>>(
        P, R, W.lens, Qs, W.n_tab, T, W.la[0], c->lens_interval, c->lens_service);
    CT_CUDA(cudaGetLastError());
    ++launches;
    for (int t = 0; t < W.n_tab; ++t) {  // the molecules' ends, in full warps
      finish_kernel(kModeSweep)<<<c->sm_count * 8, kFinishThreads, 0, s>>>(P, R, W.lens, Qs.q[t], Qs.q[t],
                                                                          W.done[t], W.done_cap[t]);
      CT_CUDA(cudaGetLastError());
      ++launches;
    }
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
    // the force kappa_c W'(E) (kappa_c = -2 alpha_c / m) points away from the
    // axis for every configuration when no alpha_c is negative and every
    // table's slope W'(E) <= 0 (at its intervals' quarter points, up to 1e-5
    // of its largest): the entrant order then bounds steps by free flight
    bool out = true;
    for (int k = 0; k < n_cfg && out; ++k) out = sw->alpha[k] >= 0.0;
    for (int t = 0; t < W.n_tab && out; ++t) {
      const HostTable& ht = c->tables[tab_id[t]];
      const double h = (ht.knots[ht.n - 1] - ht.knots[0]) / double(ht.n - 1);
      double wmax = 0.0;
      for (int j = 0; j < ht.n - 1; ++j) wmax = std::max(wmax, std::fabs(ht.coef[size_t(j) * 4 + 2]));
      for (int j = 0; j < ht.n - 1 && out; ++j) {
        const double* cj = &ht.coef[size_t(j) * 4];
        for (int q = 0; q <= 4 && out; ++q) {
          const double u = 0.25 * q;
          out = cj[2] + u * (2.0 * cj[1] * h + u * 3.0 * cj[0] * h * h) <= 1e-5 * wmax;
        }
      }
    }
    W.outward = out ? 1 : 0;
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
    // end records for the first eighth of each table's queue (at least 2^20
    // positions): the lens entrants are a few percent of the molecules; the
    // pass ends any molecule beyond that itself
    size_t recs = 0, dcap[CTRAJ_MAX_TABLES];
    for (int t = 0; t < W.n_tab; ++t) {
      const size_t qcap = size_t(std::max<int64_t>(tab_n[t], 1));
      dcap[t] = std::min(qcap, std::max<size_t>(size_t(1) << 20, qcap / 8));
      recs += dcap[t];
    }
    if ((st = ens(c->sweep_done, recs * kDoneRecBytes))) return st;
    size_t o = 0;
    for (int t = 0; t < W.n_tab; ++t) {
      W.done[t] = reinterpret_cast<DoneRec*>(c->sweep_done.as<char>() + o * kDoneRecBytes);
      W.done_cap[t] = unsigned(dcap[t]);
      o += dcap[t];
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
  W.threads = W.force == kForceStark2Lin && sweep_staged(W) ? c->lens_threads : kPersistThreads;

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
  put(&c->lens_service, sizeof c->lens_service);
  put(&c->front_threads, sizeof c->front_threads);
  put(&W.force, sizeof W.force);
  put(&W.outward, sizeof W.outward);
  put(&W.threads, sizeof W.threads);
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
    CT_CUDA(cudaFuncSetAttribute(sweep_persist_kernel(W.force, sweep_staged(W), W.threads),
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(sweep_persist_smem(W))));
  CT_CUDA(cudaFuncSetAttribute(k_sweep_front<Mol32<false, false>>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(sweep_front_smem(kFrontMaxThreads))));
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

