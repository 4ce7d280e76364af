// libctraj.so: the soft transmission and its discrete adjoint
// (ctraj_soft_transmission, declared in include/ctraj.h; kernels in adjoint.cuh).
#include "adjoint.cuh"
#include "engine.h"

using namespace ctraj;

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
  if (a->aperture >= n_el || (a->aperture >= 0 && c->elements[a->aperture].type != CTRAJ_CIRCULAR_APERTURE))
    return fail(CTRAJ_EINVAL, "soft transmission: element %d is not a circular aperture", a->aperture);
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
  int npost = 0;  // circular apertures behind the lens: soft tests at both planes
  for (int i = li + 1; i < n_el; ++i) {
    const ctraj_element& e = c->elements[i];
    if (e.type != CTRAJ_CIRCULAR_APERTURE)
      return fail(CTRAJ_EINVAL, "soft transmission: element %d behind the lens is not a circular aperture", i);
    const double r = i == a->aperture ? prm[CTRAJ_SOFT_APERTURE_R] : e.p[0] * 0.5;
    for (int k = 0; k < 2; ++k) {
      S.post_z[npost] = k ? e.z1 : e.z0;
      S.post_radius[npost] = std::isinf(r) ? INFINITY : r;
      S.post_param[npost] = i == a->aperture;
      ++npost;
    }
  }
  S.n_post = npost;
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
  const int tid = c->elements[li].table;
  const HostTable& t = c->tables[tid];
  const double h = (t.knots[t.n - 1] - t.knots[0]) / double(t.n - 1);
  const size_t tb = size_t(t.n - 1) * sizeof(Coef4<T>);
  if (tb > 200 * 1024) return fail(CTRAJ_EINVAL, "soft transmission: the lens table (%d knots) is too large", t.n);
  int st;
  // table f W'(E) = q0 + q1 u + q2 u^2 on each interval, in T, with a power of
  // two f that brings the largest coefficient near 1 (W' is ~1e-29 J m/V and
  // kappa beta ~1e40 would overflow float); kappa and kappa1 carry 1/f.  It
  // depends on the Stark table alone, not on the parameters: built and
  // uploaded again only when the table (or anything set since) changed, so a
  // gradient loop does not rebuild it per call.
  if (c->soft_table_gen != c->generation || c->soft_table_id != tid || c->soft_table_size != int(sizeof(T))) {
    double qmax = 0.0;
    for (int j = 0; j < t.n - 1; ++j) {
      const double* cj = &t.coef[size_t(j) * 4];
      qmax = std::max({qmax, std::fabs(cj[2]), std::fabs(2.0 * cj[1] * h), std::fabs(3.0 * cj[0] * h * h)});
    }
    const double f = qmax > 0.0 && std::isfinite(qmax) ? std::ldexp(1.0, -std::ilogb(qmax)) : 1.0;
    std::vector<Coef4<T>> host(t.n - 1);
    for (int j = 0; j < t.n - 1; ++j) {
      const double* cj = &t.coef[size_t(j) * 4];
      host[j] = Coef4<T>{T(f * cj[2]), T(f * (2.0 * cj[1] * h)), T(f * (3.0 * cj[0] * h * h)), T(0)};
    }
    c->soft_table_gen = ~uint64_t(0);  // until the copy is enqueued
    if ((st = c->soft_table.ensure(tb))) return st;
    CT_CUDA(cudaMemcpyAsync(c->soft_table.p, host.data(), tb, cudaMemcpyHostToDevice, s));
    CT_CUDA(cudaStreamSynchronize(s));  // host goes out of scope
    c->soft_table_gen = c->generation;
    c->soft_table_id = tid;
    c->soft_table_size = int(sizeof(T));
    c->soft_table_f = f;
  }
  S.kappa /= c->soft_table_f;
  S.kappa1 /= c->soft_table_f;
  const int64_t chunk = std::min<int64_t>(std::max<int64_t>(a->n, 1), kSoftChunk);
  if ((st = c->soft_queue.ensure(size_t(chunk) * 4 * 3))) return st;
  if ((st = c->soft_ctl.ensure(kSoftCtlBytes))) return st;
  if ((st = c->soft_contrib.ensure(size_t(chunk) * kSoftAcc * 8))) return st;
  const bool post_grad = a->want_grad && S.n_post > 0;
  if (a->ic_mode == CTRAJ_IC_HOST && a->n > 0) {
    const size_t b = size_t(a->n) * 5 * 8;
    if ((st = c->ics.ensure(b))) return st;
    CT_CUDA(cudaMemcpyAsync(c->ics.p, a->normals, b, cudaMemcpyHostToDevice, s));
    S.normals = c->ics.as<double>();
  }
  SoftQueue Q{c->soft_queue.as<int32_t>(), c->soft_ctl.as<unsigned>(0), c->soft_ctl.as<unsigned>(4),
              c->soft_queue.as<int32_t>(size_t(chunk) * 4), c->soft_queue.as<int32_t>(size_t(chunk) * 8),
              c->soft_ctl.as<unsigned>(8), nullptr};
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
      if (post_grad) {
        if ((st = c->soft_post.ensure(5 * cap * sizeof(double), 25))) return st;
        Q.bpost = c->soft_post.as<double>();
      }
      if (a->want_grad) {
        if ((st = c->soft_ckpt.ensure(n_seg * 8 * cap * sizeof(T), 25))) return st;
        if ((st = c->soft_seg.ensure(size_t(kSoftSegStride) * cap * size_t(max_seg) * sizeof(T), 25))) return st;
      }
      grid = int((cap + kSoftThreads - 1) / kSoftThreads);
      kl<<<grid, kSoftThreads, tb, s>>>(S, Q, c->soft_table.as<Coef4<T>>(), c->soft_ckpt.as<T>(), cap, contrib,
                                         stats);
      CT_CUDA(cudaGetLastError());
      ++launches;
      if (a->want_grad) {
        // backward: every (survivor, segment) in parallel, then per survivor
        // the composition and the ballistic part (also when no molecule took
        // a lens step); both read the survivor count on the device
        if (max_seg > 0) {
          auto ks = k_soft_seg<T>;
          CT_CUDA(cudaFuncSetAttribute(ks, cudaFuncAttributeMaxDynamicSharedMemorySize, int(tb)));
          const int gs = blocks_per_sm(ks, kSoftThreads, tb) * c->sm_count * 4;
          ks<<<gs, kSoftThreads, tb, s>>>(S, Q, c->soft_table.as<Coef4<T>>(), c->soft_ckpt.as<T>(), cap,
                                          c->soft_seg.as<T>(), max_seg);
          CT_CUDA(cudaGetLastError());
          ++launches;
        }
        k_soft_compose<T><<<grid, kSoftThreads, 0, s>>>(S, Q, c->soft_seg.as<T>(), max_seg, contrib, cap);
        CT_CUDA(cudaGetLastError());
        ++launches;
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

