// Propagation kernels.
//
// One run = k_front over all molecules, then, for each electrostatic lens in
// beamline order, k_lens_chunk launched until the lens is empty.
//
// k_front (one thread per molecule, grid-stride): draws or loads the initial
//   conditions, walks the ballistic elements in closed form and stops at the
//   first lens entrance.  Molecules lost on the way (98 % on the lens-beamline
//   workload) are tallied at once; molecules inside the lens bore get their
//   step count, step size and exit-snap time (in double) and are staged in
//   shared memory (ballot + prefix popcount per warp), then appended to a
//   queue by the CTA with one atomic per flush: the stream compaction between
//   element segments.
// k_lens_chunk (one thread per queued molecule, the lens's table staged in
//   shared memory per CTA): at most `chunk` RK4 steps per molecule, then the
//   molecules still inside the lens are compacted into the next chunk's
//   queue.  Every chunk therefore starts with full warps although molecules
//   are lost at very different steps.  Molecules that leave the lens do the
//   exit snap and the ballistic elements after it here, then are tallied or
//   queued at the next lens.
// k_lens_persist (FP32 runs): the whole lens in one launch, lanes refilled
//   from the queue as their molecules finish, the last molecules compacted
//   into few warps (see the kernel); k_lens_chunk remains the path for FP64,
//   ring recording and batched sweeps.
// k_record: replays chosen molecules one thread each and writes their
//   trajectory rows (trajectory recording for apertures of interest).
//
// Tallies: each warp combines equal labels with __match_any_sync and adds the
// popcount to a shared-memory counter; each CTA flushes its counters to global
// memory once (integer atomics, so the totals do not depend on order).
#pragma once
#include "molecule.cuh"

namespace ctraj {


constexpr unsigned kFull = 0xffffffffu;
constexpr int kThreads = 256;
constexpr int kFrontMaxThreads = 512;  // k_front is launched with 128-512 threads (tuning)
constexpr int kFrontSlack = 64;        // k_front: staging entries beyond one per thread
// Lens chunks: 512 threads, 2 CTAs per SM (<= 64 registers): 32 warps share
// two copies of the staged table (2 x 64 KiB for 4096 knots).
constexpr int kLensThreads = 512;

struct BlockTally {
  unsigned long long cnt[CTRAJ_MAX_LABELS + 1];
  unsigned long long stat[kStatCount];
};

__device__ __forceinline__ void tally_init(BlockTally& S) {
  for (int k = threadIdx.x; k < CTRAJ_MAX_LABELS + 1; k += blockDim.x) S.cnt[k] = 0;
  for (int k = threadIdx.x; k < kStatCount; k += blockDim.x) S.stat[k] = 0;
}

// all 32 lanes must call this together
__device__ __forceinline__ void tally_warp(BlockTally& S, int label, int n_labels) {
  const unsigned peers = __match_any_sync(kFull, label);
  const int lane = threadIdx.x & 31;
  if (label != kNone && label != kQueued && lane == __ffs(peers) - 1) {
    const int slot = label < 0 ? n_labels : label;
    atomicAdd(&S.cnt[slot], (unsigned long long)__popc(peers));
  }
}

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
  return v;
}

// all 32 lanes must call this together
__device__ __forceinline__ void stat_add(BlockTally& S, int k, unsigned long long v) {
  v = warp_sum(v);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(&S.stat[k], v);
}

// Per-configuration tallies of a batched sweep (all 32 lanes call): lanes with
// equal (configuration, label) are combined, one global atomic per group.
__device__ __forceinline__ void tally_cfg(const RunDev& R, int cfg, int label, int n_labels) {
  const bool counted = label != kNone && label != kQueued;
  const int key = counted ? cfg * (n_labels + 1) + (label < 0 ? n_labels : label) : -1;
  const unsigned peers = __match_any_sync(kFull, key);
  if (counted && (threadIdx.x & 31) == __ffs(peers) - 1)
    atomicAdd(&R.cfg_counts[key], (unsigned long long)__popc(peers));
}

// Configuration of sweep molecule i: the last c with cfg_start[c] <= i.
__device__ __forceinline__ int find_cfg(const RunDev& R, int64_t i) {
  int lo = 0, hi = R.n_cfg - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(R.cfg_start + mid) <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// Per-run stats of a grouped batch (all 32 lanes call; run < 0: nothing to
// add): lanes of the same run are combined, one global atomic per run and
// nonzero stat.  Sums fit in 32 bits per warp (steps of one molecule < 2^26).
__device__ __forceinline__ void stats_run(const RunDev& R, int run, const unsigned (&v)[kStatMaxSteps]) {
  const unsigned peers = __match_any_sync(kFull, run);
  const bool leader = run >= 0 && (threadIdx.x & 31) == __ffs(peers) - 1;
#pragma unroll
  for (int k = 0; k < kStatMaxSteps; ++k) {
    const unsigned t = __reduce_add_sync(peers, v[k]);
    if (leader && t) atomicAdd(&R.cfg_stats[size_t(run) * kStatCount + k], (unsigned long long)t);
  }
}

__device__ __forceinline__ void tally_flush(BlockTally& S, const RunDev& R, int n_labels) {
  __syncthreads();
  for (int k = threadIdx.x; k <= n_labels; k += blockDim.x)
    if (S.cnt[k]) atomicAdd(&R.counts[k], S.cnt[k]);
  for (int k = threadIdx.x; k < kStatCount; k += blockDim.x)
    if (S.stat[k]) atomicAdd(&R.stats[k], S.stat[k]);
}

// Reserve queue slots for the lanes with push == true (all lanes call).
__device__ __forceinline__ unsigned queue_slot(bool push, unsigned* count) {
  const unsigned m = __ballot_sync(kFull, push);
  const int lane = threadIdx.x & 31;
  unsigned base = 0;
  if (m) {
    const int leader = __ffs(m) - 1;
    if (lane == leader) base = atomicAdd(count, unsigned(__popc(m)));
    base = __shfl_sync(kFull, base, leader);
  }
  return base + unsigned(__popc(m & ((1u << lane) - 1u)));
}

template <class M, bool kOut>
__device__ __forceinline__ void write_outputs(const RunDev& R, const M& m, int label) {
  if (!kOut) return;
  const int64_t i = m.id;
  if (R.out_label) R.out_label[i] = label;
  if (R.out_rows) R.out_rows[i] = m.rows;
  if (R.out_margin) R.out_margin[i] = double(m.margin);
  if (R.out_final) m.final_row(R.out_final, i, R.n);
}


// Step parameters of a molecule that passed the entrance of lens `li`; false
// when rint(L/dz) is not finite or too large (the reference raises there).
template <class M>
__device__ __forceinline__ bool enter_lens(M& m, const Plan& P, int li, LensStep& st) {
  if (!lens_setup(P.el[li], m.vel_z(), st)) return false;
  m.lens_begin(P, li, st);
  return true;
}

// FP32 runs leave the exact step setup (three double divisions) of a molecule
// entering the first lens to the first lens chunk, whose warps are full; here
// only n_total = -1 ("pending") and a float upper bound on the step count,
// which sizes the chunk loop.
template <class M>
__device__ __forceinline__ bool enter_lens_front(M& m, const Plan& P, int li, LensStep& st) {
  if (!M::kDeferLensSetup) return enter_lens(m, P, li, st);
  const ctraj_element& e = P.el[li];
  const float dz = e.step_mode == CTRAJ_STEP_DT ? float(m.vel_z()) * float(e.p[2]) : float(e.p[1]);
  const float bound = fabsf(float(e.p[7]) / dz);
  st.n_done = 0;
  st.n_total = -1;
  // NaN / inf / oversize: the exact setup in the first chunk rejects the molecule
  st.bound = bound < float(CTRAJ_MAX_LENS_STEPS) ? int(bound) + 2 : int(CTRAJ_MAX_LENS_STEPS) + 1;
  return true;
}

// What push_lens stores in Queue::cfg: nothing, the given tag (a sweep's
// configuration or a carried record slot), or the slot itself (a new record
// slot for ring recording).
enum : int { kTagNone = 0, kTagCarry = 1, kTagSlot = 2 };

// Append the lanes with push == true to Q and raise Q's largest remaining
// step count (all lanes call).  Returns the lane's slot.
//
// run_max (grouped batch): where the largest step bound of this lane's run is
// kept (per lane, so lanes of different runs may push together); warp_max:
// the same for a warp whose lanes all belong to one run (one atomic).
template <int kTag = kTagNone, class M>
__device__ __forceinline__ unsigned push_lens(const Queue& Q, bool push, const M& m, const LensStep& st,
                                              int tag = 0, unsigned long long* run_max = nullptr,
                                              unsigned long long* warp_max = nullptr) {
  const unsigned slot = queue_slot(push, Q.count);
  if (push) {
    m.store(Q, slot, st);
    if (kTag == kTagCarry) Q.cfg[slot] = tag;
    if (kTag == kTagSlot) Q.cfg[slot] = int(slot);
  }
  const unsigned rem = push ? unsigned(st.n_total < 0 ? st.bound : st.n_total - st.n_done) : 0u;
  const unsigned wmax = __reduce_max_sync(kFull, rem);
  if ((threadIdx.x & 31) == 0 && wmax) {
    atomicMax(Q.max_steps, wmax);
    if (warp_max) atomicMax(warp_max, (unsigned long long)wmax);
  }
  if (run_max && rem) atomicMax(run_max, (unsigned long long)rem);
  return slot;
}

// Ring row r (mod capacity): x, y, z, vx, vy, vz, t, step.
__device__ __forceinline__ void ring_row(const ctraj_ring& G, unsigned long long r, float x, float y, float z,
                                         float vx, float vy, float vz, float t, float step) {
  float4* row = reinterpret_cast<float4*>(G.rows + size_t(r % (unsigned long long)G.capacity_rows) * 8);
  row[0] = make_float4(x, y, z, vx);
  row[1] = make_float4(vy, vz, t, step);
}

__device__ __forceinline__ void ring_entry(const ctraj_ring& G, unsigned long long m, int64_t id,
                                           unsigned long long first, int rows, int label) {
  ctraj_ring_entry en;
  en.molecule = id;
  en.first_row = first;
  en.rows = rows;
  en.label = label;
  G.index[m % (unsigned long long)G.capacity_molecules] = en;
}

// ---------------------------------------------------------------------------
// kModeRing (FP32 ring recording): the molecules queued at the recorded lens
// (the first lens) get their queue slot as record slot, and those stopped by
// its entrance test are appended to the ring at once.  kModeBatch (grouped
// batch): the lens entrants carry the run's tag R.run_tag, and the largest
// step bound queued is kept in the run's stats (counts and stats go to the
// run's own slots through R.counts / R.stats).  The block size is a launch
// parameter (at most kFrontMaxThreads).
//
// Lens entrants are staged in shared memory and appended to the queue by the
// CTA at its end, with one global atomic, instead of one returning atomic
// per warp on the queue's single counter.  The staging area holds
// front_stage(threads) entries; a warp whose entrants do not all fit appends
// the rest itself (queue_slot), so no warp waits for another before the end.
//
// Screening (FP32 runs without per-molecule outputs, device draws with a
// Gaussian position, element 0 a circular or rectangular aperture): most
// molecules of such a beamline are stopped at element 0's entrance plane by
// their x alone, which the first of a molecule's two Philox calls decides
// (Mol32::screened_out).  Those are tallied there; the others wait in a
// per-warp buffer (index, vx, vy, vz, x) and are taken 32 at a time, in full
// warps, for the second call and the walk -- the same results as the full
// walk of every molecule, with the second call, a Box-Muller pair and the
// walk's divergent work left out for the screened ones.
template <class M>
struct FrontEntry {
  M m;
  LensStep st;
};

struct ScreenSlot {
  int32_t i;
  float vx, vy, vz, x;
};
constexpr int kScreenSlots = 64;  // per warp: under 32 waiting plus one iteration's 32

__host__ __device__ constexpr unsigned front_stage(int threads) { return unsigned(threads / 2 + kFrontSlack); }

template <class M>
__host__ __device__ constexpr size_t front_smem(int threads) {
  return size_t(front_stage(threads)) * sizeof(FrontEntry<M>) +
         size_t(threads / 32) * kScreenSlots * sizeof(ScreenSlot);
}

template <class M, bool kOut, int kMode = kModePlain>
__global__ void __launch_bounds__(kFrontMaxThreads) k_front(const __grid_constant__ Plan P, const RunDev R,
                                                    const Queue Q) {
  extern __shared__ __align__(16) unsigned char s_front[];
  FrontEntry<M>* stage = reinterpret_cast<FrontEntry<M>*>(s_front);
  ScreenSlot* scr = reinterpret_cast<ScreenSlot*>(s_front + size_t(front_stage(blockDim.x)) * sizeof(FrontEntry<M>)) +
                    (threadIdx.x >> 5) * kScreenSlots;
  __shared__ BlockTally S;
  __shared__ unsigned s_n, s_base, s_max;
  tally_init(S);
  if (threadIdx.x == 0) s_n = s_max = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const unsigned lanes_lt = (1u << lane) - 1u;
  const unsigned cap = front_stage(blockDim.x);
  // the queue's (and a batch run's) largest remaining step count
  auto raise_max = [&](unsigned v) {
    atomicMax(Q.max_steps, v);
    if (kMode == kModeBatch) atomicMax(R.stats + kStatMaxSteps, (unsigned long long)v);
  };
  auto tag = [&](unsigned slot) {
    if (kMode == kModeRing) Q.cfg[slot] = int(slot);  // the record slot
    if (kMode == kModeBatch) Q.cfg[slot] = R.run_tag;
  };
  unsigned long long steps = 0, band = 0, bad = 0;
  // molecule i of this lane (i < 0: none; ready: m already drawn) through
  // the walk, the staging of lens entrants and the tally; all lanes of the
  // warp call it together
  auto one = [&](const int64_t i, M& m, const bool ready) {
    int label = kNone;
    LensStep st;
    if (i >= 0) {
      if (!ready) m.init(P, R, i);
      int lens_at = -1;
      label = walk(m, P, 0, &lens_at);
      if (label == kQueued && !enter_lens_front(m, P, lens_at, st)) {
        label = P.el[lens_at].label_inside;
        ++bad;
      }
      if (label != kQueued) {
        steps += unsigned(m.rows);
        band += (m.margin < kEdgeBand) ? 1 : 0;
        write_outputs<M, kOut>(R, m, label);
      }
      if constexpr (kMode == kModeRing) {  // listed; k_ring_reserve / k_ring_write append them
        if (label == R.rec_entrance_label && lens_at == R.rec_lens) R.ent_id[atomicAdd(R.ent_count, 1u)] = int32_t(i);
      }
    }
    // this warp's lens entrants: staged while the area has room (one shared
    // atomic per warp), the overflow appended to the queue directly
    const bool push = label == kQueued;
    const unsigned pm = __ballot_sync(kFull, push);
    if (pm) {
      unsigned wb = 0;
      if (lane == 0) wb = atomicAdd(&s_n, unsigned(__popc(pm)));
      wb = __shfl_sync(kFull, wb, 0);
      const unsigned rem = push ? unsigned(st.n_total < 0 ? st.bound : st.n_total - st.n_done) : 0u;
      const unsigned wmax = __reduce_max_sync(kFull, rem);
      const unsigned pos = wb + __popc(pm & lanes_lt);
      const bool over = push && pos >= cap;
      if (push && !over) {
        FrontEntry<M>& e = stage[pos];
        e.m = m;
        e.st = st;
      }
      if (wb + unsigned(__popc(pm)) <= cap) {  // warp-uniform: all staged
        if (lane == 0 && wmax) atomicMax(&s_max, wmax);
      } else {
        const unsigned slot = queue_slot(over, Q.count);
        if (over) {
          m.store(Q, slot, st);
          tag(slot);
        }
        if (lane == 0 && wmax) raise_max(wmax);
      }
    }
    tally_warp(S, label, P.n_labels);
  };
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  const int64_t first = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31);  // warp-uniform loops
  bool screen = false;
  if constexpr (M::kScreenable) {
    const ctraj_element& e0 = P.el[0];
    screen = R.ic_mode == CTRAJ_IC_DEVICE_DRAW && R.xd.kind != CTRAJ_DIST_DISC_POSITION &&
             isfinite(float(R.xd.p[1])) && P.n_el > 0 &&
             (e0.type == CTRAJ_CIRCULAR_APERTURE || e0.type == CTRAJ_RECTANGULAR_APERTURE);
  }
  if (screen) {
    if constexpr (M::kScreenable) {
      int waiting = 0;  // warp-uniform: molecules in this warp's buffer
      // the last k waiting molecules, one per lane, through the walk
      auto take = [&](const int k) {
        M m;
        int64_t i = -1;
        if (lane < k) {
          const ScreenSlot e = scr[waiting - k + lane];
          i = e.i;
          m.vx = e.vx;
          m.vy = e.vy;
          m.vz = e.vz;
          m.x = e.x;
          m.screen_rest(P, R, i);
        }
        __syncwarp();
        waiting -= k;
        one(i, m, true);
      };
      const int label0 = P.el[0].label;
      for (int64_t base = first; base < R.n; base += stride) {
        const int64_t i = base + lane;
        M m;
        bool wait = false;
        int label = kNone;
        if (i < R.n) {
          m.screen_draw(R, i);
          if (m.screened_out(P, R.gap0f)) {
            label = label0;
            steps += 1;  // the walk's one row: the flight to element 0
          } else {
            wait = true;
          }
        }
        const unsigned wm = __ballot_sync(kFull, wait);
        if (wait) scr[waiting + __popc(wm & lanes_lt)] = ScreenSlot{int32_t(i), m.vx, m.vy, m.vz, m.x};
        waiting += __popc(wm);
        tally_warp(S, label, P.n_labels);
        __syncwarp();
        if (waiting >= 32) take(32);
      }
      while (waiting > 0) take(min(waiting, 32));
    }
  } else {
    for (int64_t base = first; base < R.n; base += stride) {
      const int64_t i = base + lane;
      M m;
      one(i < R.n ? i : -1, m, false);
    }
  }
  // the staged entrants to the queue
  __syncthreads();
  const unsigned n_staged = min(s_n, cap);
  if (threadIdx.x == 0) {
    s_base = n_staged ? atomicAdd(Q.count, n_staged) : 0u;
    if (s_max) raise_max(s_max);
  }
  __syncthreads();
  for (unsigned j = threadIdx.x; j < n_staged; j += blockDim.x) {
    const unsigned slot = s_base + j;
    stage[j].m.store(Q, slot, stage[j].st);
    tag(slot);
  }
  stat_add(S, kStatSteps, steps);
  stat_add(S, kStatEdgeBand, band);
  stat_add(S, kStatBadSteps, bad);
  tally_flush(S, R, P.n_labels);
}

// Batched sweep front: k_front over the molecules of all configurations; the
// lens entrants of configuration c go to the queue of its Stark table
// (cfg_table[c]), and every tally is also kept per configuration.  The sweep
// beamline has one lens, so a molecule queued here is at that lens.
template <class M>
__global__ void __launch_bounds__(kFrontMaxThreads) k_sweep_front(const __grid_constant__ Plan P, const RunDev R,
                                                          const __grid_constant__ SweepQueues Qs,
                                                          const int n_tables) {
  // the screening buffers of k_front (one per warp), with the configuration
  extern __shared__ __align__(16) unsigned char s_sweep[];
  ScreenSlot* scr = reinterpret_cast<ScreenSlot*>(s_sweep) + (threadIdx.x >> 5) * kScreenSlots;
  int* scr_cfg = reinterpret_cast<int*>(s_sweep + size_t(blockDim.x / 32) * kScreenSlots * sizeof(ScreenSlot)) +
                 (threadIdx.x >> 5) * kScreenSlots;
  __shared__ BlockTally S;
  tally_init(S);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const unsigned lanes_lt = (1u << lane) - 1u;
  unsigned long long steps = 0, bad = 0;
  // molecule i (configuration cfg) of this lane through the walk, its Stark
  // table's lens queue and the tallies (i < 0: none; ready: m already drawn)
  auto one = [&](const int64_t i, const int cfg, M& m, const bool ready) {
    int label = kNone, tab = -1;
    LensStep st;
    if (i >= 0) {
      tab = __ldg(R.cfg_table + cfg);
      if (!ready) m.init(P, R, i);
      int lens_at = -1;
      label = walk(m, P, 0, &lens_at);
      if (label == kQueued && !enter_lens_front(m, P, lens_at, st)) {
        label = P.el[lens_at].label_inside;
        ++bad;
      }
      if (label != kQueued) steps += unsigned(m.rows);
    }
    for (int t = 0; t < n_tables; ++t) push_lens<kTagCarry>(Qs.q[t], label == kQueued && tab == t, m, st, cfg);
    tally_warp(S, label, P.n_labels);
    tally_cfg(R, cfg, label, P.n_labels);
  };
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  const int64_t first = int64_t(blockIdx.x) * blockDim.x + (threadIdx.x & ~31);  // warp-uniform loops
  bool screen = false;
  if constexpr (M::kScreenable) {
    const ctraj_element& e0 = P.el[0];
    screen = R.ic_mode == CTRAJ_IC_DEVICE_DRAW && R.xd.kind != CTRAJ_DIST_DISC_POSITION &&
             isfinite(float(R.xd.p[1])) && P.n_el > 0 &&
             (e0.type == CTRAJ_CIRCULAR_APERTURE || e0.type == CTRAJ_RECTANGULAR_APERTURE);
  }
  if (screen) {
    if constexpr (M::kScreenable) {
      int waiting = 0;  // warp-uniform
      auto take = [&](const int k) {  // the last k waiting molecules, one per lane
        M m;
        int64_t i = -1;
        int cfg = 0;
        if (lane < k) {
          const ScreenSlot e = scr[waiting - k + lane];
          cfg = scr_cfg[waiting - k + lane];
          i = e.i;
          m.vx = e.vx;
          m.vy = e.vy;
          m.vz = e.vz;
          m.x = e.x;
          m.screen_rest(P, R, i);
        }
        __syncwarp();
        waiting -= k;
        one(i, cfg, m, true);
      };
      const int label0 = P.el[0].label;
      for (int64_t base = first; base < R.n; base += stride) {
        const int64_t i = base + lane;
        M m;
        bool wait = false;
        int label = kNone, cfg = 0;
        if (i < R.n) {
          cfg = find_cfg(R, i);
          m.screen_draw(R, i);
          if (m.screened_out(P, R.gap0f)) {
            label = label0;
            steps += 1;  // the walk's one row: the flight to element 0
          } else {
            wait = true;
          }
        }
        const unsigned wm = __ballot_sync(kFull, wait);
        if (wait) {
          const int at = waiting + __popc(wm & lanes_lt);
          scr[at] = ScreenSlot{int32_t(i), m.vx, m.vy, m.vz, m.x};
          scr_cfg[at] = cfg;
        }
        waiting += __popc(wm);
        tally_warp(S, label, P.n_labels);
        tally_cfg(R, cfg, label, P.n_labels);
        __syncwarp();
        if (waiting >= 32) take(32);
      }
      while (waiting > 0) take(min(waiting, 32));
    }
  } else {
    for (int64_t base = first; base < R.n; base += stride) {
      const int64_t i = base + lane;
      M m;
      one(i < R.n ? i : -1, i < R.n ? find_cfg(R, i) : 0, m, false);
    }
  }
  stat_add(S, kStatSteps, steps);
  stat_add(S, kStatBadSteps, bad);
  tally_flush(S, R, P.n_labels);
}

// Dynamic shared memory of k_sweep_front (the screening buffers).
__host__ __device__ constexpr size_t sweep_front_smem(int threads) {
  return size_t(threads / 32) * kScreenSlots * (sizeof(ScreenSlot) + sizeof(int));
}

// ---------------------------------------------------------------------------
enum : int { kIdle = 0, kRun = 1, kLost = 2, kExit = 3, kBad = 4 };

// kSweep (batched sweeps, FP32 only): every molecule carries its configuration;
// the staged table is unscaled and the configuration's beta and kappa scale it;
// tallies are also kept per configuration.
// kRing (ring recording, FP32 only): in the recorded lens every molecule
// carries its record slot and stages (x, y, vx, vy) at its entrance, after
// every rec_stride-th step and where it is lost; k_ring_gather appends the
// records of the molecules lost inside to the ring.
template <class M, bool kOut, int F, bool k64, bool kStaged, bool kSweep = false, bool kRing = false>
__global__ void __launch_bounds__(kLensThreads, 2) k_lens_chunk(const __grid_constant__ Plan P, const RunDev R,
                                                         const int li, const Queue Qin,
                                                         const Queue Qcont, const Queue Qnext,
                                                         const int chunk, const LensArgs L) {
  extern __shared__ float4 s_tab[];
  __shared__ BlockTally S;
  const unsigned n_in = *(volatile unsigned*)Qin.count;
  if (n_in == 0) return;
  const int lane = threadIdx.x & 31;
  // Each warp's first batch of 32 entries is fixed, interleaved across CTAs
  // (batch k -> CTA k mod grid) so that a short queue spreads over all SMs;
  // later batches come from a shared counter, so warps whose molecules are
  // lost early take more and no CTA waits on a partial second wave.  A CTA
  // that gets nothing leaves before staging the table.
  const unsigned static_entries = gridDim.x * (blockDim.x / 32) * 32u;
  auto fetch = [&]() {
    unsigned b = 0;
    if (lane == 0) b = atomicAdd(Qin.head, 32u);
    return static_entries + __shfl_sync(kFull, b, 0);
  };
  unsigned base = ((threadIdx.x >> 5) * gridDim.x + blockIdx.x) * 32u;
  tally_init(S);
  if (!__syncthreads_or(base < n_in)) return;
  if (!k64 && kStaged)
    for (int k = threadIdx.x; k < L.n_int; k += blockDim.x) s_tab[k] = __ldg(L.q + k);
  __syncthreads();

  const ctraj_element& e = P.el[li];
  const bool classic = e.scheme == CTRAJ_RK4_CLASSIC;
  unsigned long long steps = 0, lsteps = 0, band = 0, bad = 0, range = 0, rerr = 0;
  for (; base < n_in; base = fetch()) {
    const unsigned idx = base + lane;
    M m;
    LensStep st, nst;
    st.n_done = 0;
    int phase = kIdle;
    unsigned flags = 0;
    float dt = 0.f, hdt = 0.f, c2 = 0.f, dt6 = 0.f, dt26 = 0.f;
    int n0 = 0, cfg = 0;
    float beta = 0.f, kappa = 0.f;
    bool fresh = false;
    int tag = 0, to_rec = 0;
    const bool rec_on = kRing && li == R.rec_lens;
    if (idx < n_in) {
      m.load_state(Qin, idx, P, st);
      if (kSweep) {
        const int c = Qin.cfg[idx];
        beta = __ldg(R.cfg_beta + c);
        kappa = __ldg(R.cfg_kappa + c);
      }
      if constexpr (kRing) {
        if (rec_on) {
          tag = Qin.cfg[idx];
          to_rec = R.rec_stride - st.n_done % R.rec_stride;
          if (st.n_done == 0) R.rec[size_t(tag) * R.rec_max] = make_float4(m.x, m.y, m.vx, m.vy);
        }
      }
      bool ok = true;
      fresh = st.n_total < 0;
      if (fresh) {  // step setup deferred by the front kernel
        m.load_vz(Qin, idx);
        ok = enter_lens(m, P, li, st);
      }
      n0 = st.n_done;
      dt = float(st.dt);
      hdt = 0.5f * dt;
      c2 = classic ? hdt : dt;
      dt6 = dt * (1.0f / 6.0f);
      dt26 = float(st.dt * st.dt / 6.0);
      phase = !ok ? kBad : (st.n_done < st.n_total ? kRun : kExit);
    }
    for (int k = 0; k < chunk; ++k) {
      if (phase == kRun) {
        bool lost;
        if constexpr (k64) {
          int rg = 0, er = 0;
          lost = m.lens_step(P, li, st, rg, er);
          flags |= (rg ? 1u : 0u) | (er ? 2u : 0u);
        } else {
          lost = m.template lens_step<F, kStaged, kSweep>(L, dt, hdt, c2, dt6, dt26, s_tab, flags, beta,
                                                          kappa);
          if (F == kForceRadial && (flags & 2u)) lost = true;
        }
        ++st.n_done;
        m.lens_row(P, li, st);
        if constexpr (kRing) {
          if (rec_on && --to_rec == 0) {
            to_rec = R.rec_stride;
            R.rec[size_t(tag) * R.rec_max + st.n_done / R.rec_stride] = make_float4(m.x, m.y, m.vx, m.vy);
          }
        }
        if (lost) phase = kLost;
        else if (st.n_done == st.n_total) phase = kExit;
      }
      if ((k & 15) == 15 && !__any_sync(kFull, phase == kRun)) break;
    }
    asm volatile("" ::: "memory");  // keep the loads below after the loop (register pressure)
    if (idx < n_in) {
      m.load_rest(Qin, idx, st, !fresh);
      if (kSweep) cfg = Qin.cfg[idx];
    }
    if constexpr (kRing) {
      if (rec_on && idx < n_in && phase != kRun) {
        int n_rec = 0;
        if (phase == kLost) {  // the state after the losing step closes the record
          const int s = R.rec_stride, k = st.n_done;
          if (k % s != 0) R.rec[size_t(tag) * R.rec_max + k / s + 1] = make_float4(m.x, m.y, m.vx, m.vy);
          n_rec = k / s + 1 + (k % s != 0 ? 1 : 0);
          R.rec_last[tag] = k;
        }
        R.rec_n[tag] = n_rec;  // 0: left the lens (or unusable step count), not recorded
      }
      if (rec_on && idx < n_in && fresh) {
        R.rec_id[tag] = m.id;
        R.rec_t0[tag] = m.t;
        R.rec_vz[tag] = m.vz;
      }
    }
    lsteps += unsigned(st.n_done - n0);
    int label = kNone;
    bool enter = false;
    if (phase == kBad) {  // rint(L/dz) not usable: the reference raises here
      label = e.label_inside;
      ++bad;
      steps += unsigned(m.rows);
      write_outputs<M, kOut>(R, m, label);
    } else if (phase == kLost || phase == kExit) {
      range += (flags & 1u) ? 1 : 0;
      rerr += (flags & 2u) ? 1 : 0;
      m.lens_end(P, li, st, phase == kLost);
      if (phase == kLost) {
        label = e.label_inside;
      } else {
        int lens_at = -1;
        label = walk(m, P, li + 1, &lens_at);
        if (label == kQueued) {
          enter = enter_lens(m, P, lens_at, nst);
          if (!enter) {
            label = P.el[lens_at].label_inside;
            ++bad;
          }
        }
      }
      if (label != kQueued) {
        steps += unsigned(m.rows);
        band += (m.margin < double(kEdgeBand)) ? 1 : 0;
        write_outputs<M, kOut>(R, m, label);
      }
    }
    push_lens<(kSweep || kRing) ? kTagCarry : kTagNone>(Qcont, phase == kRun, m, st, kRing ? tag : cfg);
    push_lens<(kSweep || kRing) ? kTagCarry : kTagNone>(Qnext, enter, m, nst, kRing ? tag : cfg);
    tally_warp(S, label, P.n_labels);
    if (kSweep) tally_cfg(R, cfg, label, P.n_labels);
  }
  stat_add(S, kStatSteps, steps);
  stat_add(S, kStatLensSteps, lsteps);
  stat_add(S, kStatEdgeBand, band);
  stat_add(S, kStatBadSteps, bad);
  stat_add(S, kStatTableRange, range);
  stat_add(S, kStatRangeError, rerr);
  tally_flush(S, R, P.n_labels);
}

// ---------------------------------------------------------------------------
// Lens-entrant order for k_lens_persist: longest step count first.  In a lens
// pass the molecules that need the most RK4 steps (the slowest, ~5000 steps
// at dt = 1 us) form the critical path; taking them first starts that path
// at once.  A counting sort on L / dz in kOrderBuckets buckets, three
// launches: count, exclusive scan (one block), place.  The order changes no
// result: molecules are independent and tallies are integer sums.
constexpr int kOrderBuckets = 1024;

// bucket 0 = most steps, for a queue whose largest step count is max_steps.
// outward (a lens whose force points away from the axis everywhere, the
// defocused high-field seekers): such a lens loses a molecule no later than
// free flight would carry it to the bore radius R, so its steps are at most
// t vz / dz with |(x, y) + (vx, vy) t| = R -- the molecules the lens loses
// early go last, and those that cross it first, whatever their speed.  The
// key only orders the work; it changes no result.
__device__ __forceinline__ int order_bucket(const ctraj_element& e, const Queue& Q, const unsigned j,
                                            const float scale, const int outward) {
  const float vz = Q.vz[j];
  const float dz = e.step_mode == CTRAJ_STEP_DT ? fabsf(vz) * float(e.p[2]) : float(e.p[1]);
  float steps = float(e.p[7]) / dz;
  if (outward) {
    const float x = Q.x[j], y = Q.y[j], vx = Q.vx[j], vy = Q.vy[j], R = 0.5f * float(e.p[0]);
    const float a = vx * vx + vy * vy, b = x * vx + y * vy, c = x * x + y * y - R * R;
    const float t = (sqrtf(fmaxf(b * b - a * c, 0.0f)) - b) / a;  // a = 0: inf or NaN, no bound
    steps = fminf(steps, t * fabsf(vz) / dz);
  }
  const float u = float(kOrderBuckets - 1) - steps * scale;  // NaN, -inf -> 0
  return u > 0.0f ? (u < float(kOrderBuckets - 1) ? int(u) : kOrderBuckets - 1) : 0;
}

__device__ __forceinline__ float order_scale(const Queue& Q) {
  return float(kOrderBuckets - 1) / (float(*Q.max_steps) + 1.0f);
}

// Each block takes a contiguous range of the queue and counts it in shared
// memory first: the step counts of a beam cluster in a few buckets, where
// global atomics from every thread would serialise.
constexpr int kOrderThreads = 256;

__device__ __forceinline__ void order_range(unsigned n, unsigned& lo, unsigned& hi) {
  const unsigned per = (n + gridDim.x - 1) / gridDim.x;
  lo = min(n, blockIdx.x * per);
  hi = min(n, lo + per);
}

static __global__ void __launch_bounds__(kOrderThreads) k_order_count(const __grid_constant__ Plan P, const int li,
                                                               const Queue Q, unsigned* hist, const int outward) {
  __shared__ unsigned h[kOrderBuckets];
  for (int b = threadIdx.x; b < kOrderBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const float scale = order_scale(Q);
  unsigned lo, hi;
  order_range(*Q.count, lo, hi);
  for (unsigned j = lo + threadIdx.x; j < hi; j += blockDim.x)
    atomicAdd(h + order_bucket(P.el[li], Q, j, scale, outward), 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < kOrderBuckets; b += blockDim.x)
    if (h[b]) atomicAdd(hist + b, h[b]);
}

static __global__ void __launch_bounds__(kOrderBuckets) k_order_scan(unsigned* hist) {
  __shared__ unsigned t[kOrderBuckets];
  const int i = threadIdx.x;
  const unsigned own = hist[i];
  t[i] = own;
  __syncthreads();
  for (int o = 1; o < kOrderBuckets; o <<= 1) {
    const unsigned v = i >= o ? t[i - o] : 0u;
    __syncthreads();
    t[i] += v;
    __syncthreads();
  }
  hist[i] = t[i] - own;
}

// Same ranges as k_order_count: the block reserves its entries of every
// bucket with one global atomic per bucket, then places them with
// shared-memory atomics.
static __global__ void __launch_bounds__(kOrderThreads) k_order_place(const __grid_constant__ Plan P, const int li,
                                                               const Queue Q, unsigned* cursor, unsigned* order,
                                                               const int outward) {
  __shared__ unsigned h[kOrderBuckets];
  for (int b = threadIdx.x; b < kOrderBuckets; b += blockDim.x) h[b] = 0;
  __syncthreads();
  const float scale = order_scale(Q);
  unsigned lo, hi;
  order_range(*Q.count, lo, hi);
  for (unsigned j = lo + threadIdx.x; j < hi; j += blockDim.x)
    atomicAdd(h + order_bucket(P.el[li], Q, j, scale, outward), 1u);
  __syncthreads();
  for (int b = threadIdx.x; b < kOrderBuckets; b += blockDim.x)
    h[b] = h[b] ? atomicAdd(cursor + b, h[b]) : 0u;
  __syncthreads();
  for (unsigned j = lo + threadIdx.x; j < hi; j += blockDim.x)
    order[atomicAdd(h + order_bucket(P.el[li], Q, j, scale, outward), 1u)] = j;
}

// ---------------------------------------------------------------------------
// Persistent lens pass: one launch integrates a whole lens queue (FP32), one
// CTA per SM, 16 warps (k_lens_persist; k_sweep_persist runs it per Stark
// table of a batched sweep).
//
// Phase A (molecules left in the queue): every `service` steps a warp
// finalises its lanes whose molecule was lost or left the lens (exit snap,
// the elements after the lens, tally, next-lens queue) and refills them from
// the queue in `order`, so lanes stay busy while work remains.
// Phase B (queue empty): every `interval` steps the CTA counts its molecules
// and, when they fit in fewer warps, moves them through shared memory into
// the lowest warps.  The emptied warps wait at the barrier without issuing,
// so the last, longest-lived molecules run with little contention for the
// SM's issue slots -- their step time approaches the latency of one RK4 step.
//
// The molecule state a lane carries (SwapSlot) is what the RK4 loop needs;
// the rest (t, vz, rows, id, queued margin) is read back from the queue entry
// at finalisation, as k_lens_chunk does.
struct SwapSlot {
  float4 a;  // x, y, vx, vy
  float4 b;  // cx, cy, cvx, cvy
  double dt, snap;
  int4 c;    // n_done, n_total, n0, idx
  unsigned flags, phase;
  float margin;
  int cfg;   // batched sweeps: configuration
};

constexpr int kPersistThreads = 512;
constexpr int kPersistService = 64;  // default steps between phase-A services

struct PersistAcc {
  unsigned long long steps = 0, lsteps = 0, band = 0, bad = 0, range = 0, rerr = 0;
};

// The end of a molecule's pass through lens li, after its last RK4 step (all
// lanes call; `fin`: this lane has such a molecule): the rest of its queue
// entry, the exit snap, the elements after the lens, its tally and stats, or
// its entry into the next lens's queue.  phase is kLost, kExit or kBad;
// flags the table-range bits of its steps; idx its queue position; n0 its
// step count when the pass took it; fresh: its step setup was done in this
// pass (st.snap holds the exit-snap time, not the queue).  The persistent
// pass calls it as its lanes finish, or k_lens_finish afterwards from the
// pass's DoneRec records.
template <class M, bool kOut, int kMode>
__device__ __forceinline__ void lens_finish(const Plan& P, const RunDev& R, const int li, const Queue& Qin,
                                            const Queue& Qnext, const bool fin, M& m, LensStep& st,
                                            const int phase, const unsigned flags, const unsigned idx,
                                            const int n0, const bool fresh, const int cfg, BlockTally& S,
                                            PersistAcc& acc) {
  constexpr bool kSweep = kMode == kModeSweep, kRing = kMode == kModeRing, kBatch = kMode == kModeBatch;
  constexpr int kNextTag = kMode == kModePlain ? kTagNone : kTagCarry;
  const ctraj_element& e = P.el[li];
  const bool rec_on = kRing && li == R.rec_lens;
  LensStep nst;
  int label = kNone;
  bool enter = false;
  // this lane's additions to the stats (kStat* order up to kStatRangeError)
  unsigned d[kStatMaxSteps] = {0u, 0u, 0u, 0u, 0u, 0u};
  if (fin) {
    m.load_rest(Qin, idx, st, !fresh);
    if constexpr (kRing) {
      if (rec_on) {  // close the record (the state after the losing step) before the exit snap
        int n_rec = 0;
        if (phase == kLost) {
          const int rs = R.rec_stride, k = st.n_done;
          if (k % rs != 0) R.rec[size_t(cfg) * R.rec_max + k / rs + 1] = make_float4(m.x, m.y, m.vx, m.vy);
          n_rec = k / rs + 1 + (k % rs != 0 ? 1 : 0);
          R.rec_last[cfg] = k;
        }
        R.rec_n[cfg] = n_rec;  // 0: left the lens (or unusable step count), not recorded
        if (fresh) {
          R.rec_id[cfg] = m.id;
          R.rec_t0[cfg] = m.t;
          R.rec_vz[cfg] = m.vz;
        }
      }
    }
    d[kStatLensSteps] = unsigned(st.n_done - n0);
    if (phase == kBad) {  // rint(L/dz) not usable: the reference raises here
      label = e.label_inside;
      d[kStatBadSteps] = 1;
      d[kStatSteps] = unsigned(m.rows);
      write_outputs<M, kOut>(R, m, label);
    } else {
      d[kStatTableRange] = (flags & 1u) ? 1 : 0;
      d[kStatRangeError] = (flags & 2u) ? 1 : 0;
      m.lens_end(P, li, st, phase == kLost);
      if (phase == kLost) {
        label = e.label_inside;
      } else {
        int lens_at = -1;
        label = walk(m, P, li + 1, &lens_at);
        if (label == kQueued) {
          enter = enter_lens(m, P, lens_at, nst);
          if (!enter) {
            label = P.el[lens_at].label_inside;
            d[kStatBadSteps] += 1;
          }
        }
      }
      if (label != kQueued) {
        d[kStatSteps] = unsigned(m.rows);
        d[kStatEdgeBand] = (m.margin < kEdgeBand) ? 1 : 0;
        write_outputs<M, kOut>(R, m, label);
      }
    }
  }
  if constexpr (kBatch) {
    push_lens<kNextTag>(Qnext, enter, m, nst, cfg,
                        enter ? R.cfg_stats + size_t(cfg) * kStatCount + kStatMaxSteps : nullptr);
    const bool done = label != kNone;
    stats_run(R, done ? cfg : -1, d);
    tally_cfg(R, cfg, label, P.n_labels);
  } else {
    acc.steps += d[kStatSteps];
    acc.lsteps += d[kStatLensSteps];
    acc.band += d[kStatEdgeBand];
    acc.bad += d[kStatBadSteps];
    acc.range += d[kStatTableRange];
    acc.rerr += d[kStatRangeError];
    push_lens<kNextTag>(Qnext, enter, m, nst, cfg);
    tally_warp(S, label, P.n_labels);
    if (kSweep) tally_cfg(R, cfg, label, P.n_labels);
  }
}

// lens_finish as a call of its own, for the batched sweep's pass: a sweep ends
// in the pass only the molecules beyond its end records, and inlined there
// the end's code set the pass's register count (126 at 512 threads, spills
// at 768 and 1024); called, it costs a stack frame on that cold path and the
// pass fits 79 registers at 768 threads (lens pass of the bench's sweep 17.3
// -> 16.1 ms at 768, 16.8 -> 15.8 ms at 1024 threads).
template <class M, bool kOut, int kMode>
__device__ __noinline__ void lens_finish_call(const Plan& P, const RunDev& R, const int li, const Queue& Qin,
                                              const Queue& Qnext, const bool fin, M& m, LensStep& st,
                                              const int phase, const unsigned flags, const unsigned idx,
                                              const int n0, const bool fresh, const int cfg, BlockTally& S,
                                              PersistAcc& acc) {
  lens_finish<M, kOut, kMode>(P, R, li, Qin, Qnext, fin, m, st, phase, flags, idx, n0, fresh, cfg, S, acc);
}

// A molecule's state after its last RK4 step in a persistent pass whose end
// (lens_finish) is deferred to k_lens_finish: written at its queue position,
// 64 bytes, read back coalesced.  word = phase | flags << 3 | n0 << 5.
struct __align__(16) DoneRec {
  float4 a;          // x, y, vx, vy
  float4 b;          // cx, cy, cvx, cvy: carried rounding errors
  double dt;         // lens step time (set in the pass for fresh entries)
  float ax, ay;      // stored acceleration: the exit snap's
  int n_done, n_total;
  float snap;        // exit-snap time
  unsigned word;
};
static_assert(sizeof(DoneRec) == 64, "DoneRec is four 16-byte stores");

// One CTA's share of a persistent pass over Qin.  The first static_entries
// queue positions are dealt out interleaved across CTAs (entry (w * grid +
// b) * 32 + lane to lane `lane` of warp w of CTA b); the rest are taken in
// order by the lanes that become idle.  kModeSweep: molecules carry their
// configuration (Queue::cfg), whose beta and kappa scale the unscaled table,
// and tallies are also kept per configuration.  kModeBatch: molecules carry
// their run (Queue::cfg) and every tally and stat goes to that run's slots
// (RunDev::cfg_counts, cfg_stats).  Every thread of the CTA calls it; it
// returns with all of the CTA's molecules finalised.
// The state of one molecule slot of a thread in the persistent pass.
template <class M>
struct PersistSlot {
  M m;
  LensStep st;
  int phase;
  unsigned flags;
  float dt, hdt, c2, dt6, dt26;
  int n0, cfg;  // cfg: the configuration (sweep), the record slot (ring) or the run (batch)
  float beta, kappa;
  bool fresh;
  unsigned idx;
  int to_rec;   // ring recording: steps to the next staged record
};

// kMPT: molecules per thread (1 or 2).  Each thread steps its kMPT molecules
// in turn, so a step of one has the other's independent chain to issue
// against; each slot s of a warp is finalised and refilled like a warp of
// its own, and the compaction of phase B packs molecules into the lowest
// threads' slots.  kMPT = 1 is the one-molecule pass.
template <class M, bool kOut, int F, bool kStaged, int kMode, int kT = kPersistThreads, int kMPT = 1>
__device__ __forceinline__ void persist_pass(const Plan& P, const RunDev& R, const int li, const Queue& Qin,
                                             const Queue& Qnext, const LensArgs& L, const unsigned* order,
                                             const int interval, const int service,
                                             const unsigned static_entries,
                                             const float4* s_tab, SwapSlot* s_swap, unsigned* s_wcount,
                                             BlockTally& S, PersistAcc& acc, DoneRec* done = nullptr,
                                             const unsigned done_cap = 0xFFFFFFFFu) {
  constexpr bool kSweep = kMode == kModeSweep, kRing = kMode == kModeRing;
  const unsigned n_in = *(volatile unsigned*)Qin.count;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned lanes_lt = (1u << lane) - 1u;
  const ctraj_element& e = P.el[li];
  const bool classic = e.scheme == CTRAJ_RK4_CLASSIC;
  const bool rec_on = kRing && li == R.rec_lens;

  PersistSlot<M> X[kMPT];
#pragma unroll
  for (int s = 0; s < kMPT; ++s) {
    X[s].st.n_done = 0;
    X[s].phase = kIdle;
    X[s].flags = 0;
    X[s].dt = X[s].hdt = X[s].c2 = X[s].dt6 = X[s].dt26 = 0.f;
    X[s].n0 = X[s].cfg = 0;
    X[s].beta = 0.f;
    X[s].kappa = 1.f;
    X[s].fresh = false;
    X[s].idx = 0;
    X[s].to_rec = 0;
  }

  auto derive = [&](PersistSlot<M>& x) {
    x.dt = float(x.st.dt);
    x.hdt = 0.5f * x.dt;
    x.c2 = classic ? x.hdt : x.dt;
    x.dt6 = x.dt * (1.0f / 6.0f);
    x.dt26 = float(x.st.dt * x.st.dt / 6.0);
    if (kSweep) {
      x.beta = __ldg(R.cfg_beta + x.cfg);
      x.kappa = __ldg(R.cfg_kappa + x.cfg);
    }
  };
  auto take = [&](PersistSlot<M>& x, unsigned j) {  // queue position j
    x.idx = order ? __ldg(order + j) : j;
    x.flags = 0;
    x.m.load_state(Qin, x.idx, P, x.st);
    if (kMode != kModePlain) x.cfg = Qin.cfg[x.idx];
    if constexpr (kRing) {
      if (rec_on) {  // the entrance state opens the record
        x.to_rec = R.rec_stride - x.st.n_done % R.rec_stride;
        if (x.st.n_done == 0) R.rec[size_t(x.cfg) * R.rec_max] = make_float4(x.m.x, x.m.y, x.m.vx, x.m.vy);
      }
    }
    bool ok = true;
    x.fresh = x.st.n_total < 0;
    if (x.fresh) {  // step setup deferred by the front kernel
      x.m.load_vz(Qin, x.idx);
      ok = enter_lens(x.m, P, li, x.st);
    }
    x.n0 = x.st.n_done;
    derive(x);
    x.phase = !ok ? kBad : (x.st.n_done < x.st.n_total ? kRun : kExit);
  };
  auto step = [&](PersistSlot<M>& x) {
    bool lost = x.m.template lens_step<F, kStaged, kSweep>(L, x.dt, x.hdt, x.c2, x.dt6, x.dt26, s_tab, x.flags,
                                                          x.beta, x.kappa);
    if (F == kForceRadial && (x.flags & 2u)) lost = true;
    ++x.st.n_done;
    if constexpr (kRing) {
      if (rec_on && --x.to_rec == 0) {
        x.to_rec = R.rec_stride;
        R.rec[size_t(x.cfg) * R.rec_max + x.st.n_done / R.rec_stride] = make_float4(x.m.x, x.m.y, x.m.vx, x.m.vy);
      }
    }
    if (lost) x.phase = kLost;
    else if (x.st.n_done == x.st.n_total) x.phase = kExit;
  };
  auto run = [&](int n_steps) {
    bool any = false;
#pragma unroll
    for (int s = 0; s < kMPT; ++s) any = any || X[s].phase == kRun;
    if (!__any_sync(kFull, any)) return;
#pragma unroll 2  // half the loop's own compare and branch per step: 2-4 % on the pass
    for (int k = 0; k < n_steps; ++k) {
#pragma unroll
      for (int s = 0; s < kMPT; ++s)
        if (X[s].phase == kRun) step(X[s]);
    }
  };
  // all lanes: the slot-x molecules that were lost or left the lens are
  // finished (tallied, or queued at the next lens) and the slot becomes idle;
  // with `done`, only their state is written to their DoneRec and
  // k_lens_finish finishes them after the pass in full warps.
  auto finalize = [&](PersistSlot<M>& x) {
    bool fin = x.phase == kLost || x.phase == kExit || x.phase == kBad;
    if (!__any_sync(kFull, fin)) return;
    if constexpr (!kOut && (kMode == kModePlain || kMode == kModeBatch || kMode == kModeSweep)) {
      // a batch pass always defers (its host always passes `done`); a plain
      // pass or a sweep when given `done`, a sweep for the queue positions
      // below done_cap (the records it has room for; the rest end here)
      if (kMode == kModeBatch || done) {
        const bool defer = fin && (kMode != kModeSweep || x.idx < done_cap);
        if (defer) {
          int4* r = reinterpret_cast<int4*>(done + x.idx);
          r[0] = make_int4(__float_as_int(x.m.x), __float_as_int(x.m.y), __float_as_int(x.m.vx),
                           __float_as_int(x.m.vy));
          r[1] = make_int4(__float_as_int(x.m.cx), __float_as_int(x.m.cy), __float_as_int(x.m.cvx),
                           __float_as_int(x.m.cvy));
          const long long dtb = __double_as_longlong(x.st.dt);
          r[2] = make_int4(int(dtb), int(dtb >> 32), __float_as_int(x.m.ax), __float_as_int(x.m.ay));
          r[3] = make_int4(x.st.n_done, x.st.n_total, __float_as_int(float(x.st.snap)),
                           int(unsigned(x.phase) | (x.flags & 3u) << 3 | unsigned(x.n0) << 5));
          x.phase = kIdle;
        }
        if (kMode != kModeSweep) return;
        fin = fin && !defer;
        if (!__any_sync(kFull, fin)) return;
      }
    }
    if constexpr (kMode == kModeSweep) {
      lens_finish_call<M, kOut, kMode>(P, R, li, Qin, Qnext, fin, x.m, x.st, x.phase, x.flags, x.idx, x.n0,
                                       x.fresh, x.cfg, S, acc);
      if (fin) x.phase = kIdle;
    } else if constexpr (kOut || kMode != kModeBatch) {
      lens_finish<M, kOut, kMode>(P, R, li, Qin, Qnext, fin, x.m, x.st, x.phase, x.flags, x.idx, x.n0, x.fresh,
                                  x.cfg, S, acc);
      if (fin) x.phase = kIdle;
    }
  };

  // the first static_entries queue positions, interleaved across CTAs
#pragma unroll
  for (int s = 0; s < kMPT; ++s) {
    const unsigned j = ((unsigned(s) * (kT / 32) + unsigned(warp)) * gridDim.x + blockIdx.x) * 32u + unsigned(lane);
    if (j < min(n_in, static_entries)) take(X[s], j);
  }
  // phase A
  for (bool exhausted = static_entries >= n_in && static_entries > 0; !exhausted;) {
    run(service);
    unsigned idle[kMPT], n_idle = 0;
#pragma unroll
    for (int s = 0; s < kMPT; ++s) {
      finalize(X[s]);
      idle[s] = __ballot_sync(kFull, X[s].phase == kIdle);
      n_idle += unsigned(__popc(idle[s]));
    }
    if (n_idle) {
      unsigned b = 0;
      if (lane == 0) b = atomicAdd(Qin.head, n_idle);
      b = static_entries + __shfl_sync(kFull, b, 0);
      exhausted = b + n_idle >= n_in;
#pragma unroll
      for (int s = 0; s < kMPT; ++s) {
        const unsigned j = b + unsigned(__popc(idle[s] & lanes_lt));
        if (X[s].phase == kIdle && j < n_in) take(X[s], j);
        b += unsigned(__popc(idle[s]));
      }
    } else {
      exhausted = static_entries + *(volatile unsigned*)Qin.head >= n_in;
    }
  }
  // phase B (every warp of the CTA enters it, then the barriers below match)
  for (;;) {
    run(interval);
    unsigned held = 0;  // molecules this thread holds
#pragma unroll
    for (int s = 0; s < kMPT; ++s) {
      finalize(X[s]);
      held += X[s].phase != kIdle ? 1u : 0u;
    }
    unsigned excl = held;  // exclusive prefix of held over the warp's lanes
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned v = __shfl_up_sync(kFull, excl, o);
      if (lane >= o) excl += v;
    }
    excl -= held;
    const unsigned wsum = __shfl_sync(kFull, excl + held, 31);
    if (lane == 0) s_wcount[warp] = wsum;
    __syncthreads();
    unsigned total = 0, base = 0, used = 0;
#pragma unroll
    for (int w = 0; w < kT / 32; ++w) {
      const unsigned c = s_wcount[w];
      base += w < warp ? c : 0u;
      total += c;
      used += c ? 1u : 0u;
    }
    __syncthreads();
    if (total == 0) break;
    if ((total + 32 * kMPT - 1) / (32 * kMPT) < used) {
      unsigned r = base + excl;
#pragma unroll
      for (int s = 0; s < kMPT; ++s) {
        const PersistSlot<M>& x = X[s];
        if (x.phase != kIdle) {
          SwapSlot& w = s_swap[r++];
          w.a = make_float4(x.m.x, x.m.y, x.m.vx, x.m.vy);
          w.b = make_float4(x.m.cx, x.m.cy, x.m.cvx, x.m.cvy);
          w.dt = x.st.dt;
          w.snap = x.st.snap;
          w.c = make_int4(x.st.n_done, x.st.n_total, x.n0, int(x.idx));
          w.flags = x.flags | (x.fresh ? 0x80000000u : 0u);
          w.phase = unsigned(x.phase);
          w.margin = x.m.margin;
          w.cfg = x.cfg;
        }
      }
      __syncthreads();
      // molecule q goes to slot q % kMPT of thread q / kMPT: the lowest warps fill up
#pragma unroll
      for (int s = 0; s < kMPT; ++s) {
        PersistSlot<M>& x = X[s];
        x.phase = kIdle;
        const unsigned q = threadIdx.x * kMPT + unsigned(s);
        if (q < total) {
          const SwapSlot& w = s_swap[q];
          x.m.x = w.a.x;
          x.m.y = w.a.y;
          x.m.vx = w.a.z;
          x.m.vy = w.a.w;
          x.m.cx = w.b.x;
          x.m.cy = w.b.y;
          x.m.cvx = w.b.z;
          x.m.cvy = w.b.w;
          x.st.dt = w.dt;
          x.st.snap = w.snap;
          x.st.n_done = w.c.x;
          x.st.n_total = w.c.y;
          x.n0 = w.c.z;
          x.idx = unsigned(w.c.w);
          x.flags = w.flags & 0x7fffffffu;
          x.fresh = (w.flags >> 31) != 0;
          x.phase = int(w.phase);
          x.m.margin = w.margin;
          x.cfg = w.cfg;
          if (kRing && rec_on) x.to_rec = R.rec_stride - x.st.n_done % R.rec_stride;
          derive(x);
        }
      }
      __syncthreads();
    }
  }
}

__device__ __forceinline__ void persist_flush(BlockTally& S, const RunDev& R, int n_labels, const PersistAcc& a) {
  stat_add(S, kStatSteps, a.steps);
  stat_add(S, kStatLensSteps, a.lsteps);
  stat_add(S, kStatEdgeBand, a.band);
  stat_add(S, kStatBadSteps, a.bad);
  stat_add(S, kStatTableRange, a.range);
  stat_add(S, kStatRangeError, a.rerr);
  tally_flush(S, R, n_labels);
}

// kT: threads per CTA (one CTA per SM, so kT / 32 warps per SM), a
// compile-time constant so that __launch_bounds__ gives the register budget
// of that occupancy; kMPT molecules per thread (the swap area holds kT x kMPT
// slots).
template <class M, bool kOut, int F, bool kStaged, int kMode = kModePlain, int kT = kPersistThreads, int kMPT = 1>
__global__ void __launch_bounds__(kT, 1) k_lens_persist(const __grid_constant__ Plan P, const RunDev R,
                                                        const int li, const Queue Qin, const Queue Qnext,
                                                        const LensArgs L, const unsigned* order,
                                                        const int interval, const int service, DoneRec* done) {
  extern __shared__ float4 s_dyn[];
  __shared__ BlockTally S;
  __shared__ unsigned s_wcount[kT / 32];
  SwapSlot* s_swap = reinterpret_cast<SwapSlot*>(s_dyn + (kStaged ? L.n_int : 0));
  if (*(volatile unsigned*)Qin.count == 0) return;
  tally_init(S);
  if (kStaged)
    for (int k = threadIdx.x; k < L.n_int; k += blockDim.x) s_dyn[k] = __ldg(L.q + k);
  __syncthreads();
  PersistAcc acc;
  // a short queue spreads over all SMs through the interleaved first entries
  persist_pass<M, kOut, F, kStaged, kMode, kT, kMPT>(P, R, li, Qin, Qnext, L, order, interval, service,
                                                      gridDim.x * kT * kMPT, s_dyn, s_swap, s_wcount, S, acc,
                                                      done);
  // a batch's tallies went to its runs; deferred ends are tallied by k_lens_finish
  if (kMode != kModeBatch && !done) persist_flush(S, R, P.n_labels, acc);
}

// The deferred ends of a persistent pass's molecules (lens_finish), one
// thread per queue position of Qin below `cap`, in full warps, from the
// DoneRec records the pass wrote (k_lens_persist with `done`: runs without
// per-molecule outputs, plain or batch mode; k_sweep_persist, per Stark
// table).  Grid-stride over the queue.
constexpr int kFinishThreads = 256;

template <class M, int kMode>
__global__ void __launch_bounds__(kFinishThreads) k_lens_finish(const __grid_constant__ Plan P, const RunDev R,
                                                                const int li, const Queue Qin, const Queue Qnext,
                                                                const DoneRec* done, const unsigned cap) {
  __shared__ BlockTally S;
  tally_init(S);
  __syncthreads();
  PersistAcc acc;
  const unsigned n = min(*(volatile unsigned*)Qin.count, cap);  // cap: the records written
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {  // warp-uniform
    const unsigned j = base + (threadIdx.x & 31);
    const bool fin = j < n;
    M m;
    LensStep st;
    int phase = kIdle, n0 = 0, cfg = 0;
    unsigned flags = 0;
    if (fin) {
      const int4* r = reinterpret_cast<const int4*>(done + j);
      const int4 r0 = r[0], r1 = r[1], r2 = r[2], r3 = r[3];
      m.x = __int_as_float(r0.x);
      m.y = __int_as_float(r0.y);
      m.vx = __int_as_float(r0.z);
      m.vy = __int_as_float(r0.w);
      m.cx = __int_as_float(r1.x);
      m.cy = __int_as_float(r1.y);
      m.cvx = __int_as_float(r1.z);
      m.cvy = __int_as_float(r1.w);
      st.dt = __longlong_as_double((long long)(unsigned(r2.x)) | (long long)(r2.y) << 32);
      m.ax = __int_as_float(r2.z);
      m.ay = __int_as_float(r2.w);
      st.n_done = r3.x;
      st.n_total = r3.y;
      st.snap = double(__int_as_float(r3.z));
      phase = int(unsigned(r3.w) & 7u);
      flags = (unsigned(r3.w) >> 3) & 3u;
      n0 = int(unsigned(r3.w) >> 5);
      m.margin = INFINITY;
      if (kMode != kModePlain) cfg = Qin.cfg[j];
    }
    // fresh = true: the exit-snap time comes from the record, not the queue
    lens_finish<M, false, kMode>(P, R, li, Qin, Qnext, fin, m, st, phase, flags, j, n0, true, cfg, S, acc);
  }
  if (kMode != kModeBatch) persist_flush(S, R, P.n_labels, acc);
}

// Batched sweep: the Stark tables' lens queues in one launch.  Each CTA
// starts on a table, chosen so that CTAs are spread over the tables in
// proportion to their queues, and when that queue is used up moves on to the
// next table with molecules left, staging its table.  kT threads per CTA
// (one CTA per SM).
struct SweepTabs {
  const float4* q[CTRAJ_MAX_TABLES];
  const unsigned* order[CTRAJ_MAX_TABLES];
  float s0[CTRAJ_MAX_TABLES];
  int n_int[CTRAJ_MAX_TABLES];
  DoneRec* done[CTRAJ_MAX_TABLES];         // deferred molecule ends (nullptr: none)
  unsigned done_cap[CTRAJ_MAX_TABLES];     // queue positions with a record
};

template <int F, bool kStaged, int kT = kPersistThreads>
__global__ void __launch_bounds__(kT, 1) k_sweep_persist(const __grid_constant__ Plan P, const RunDev R,
                                                                      const int li,
                                                                      const __grid_constant__ SweepQueues Qs,
                                                                      const int n_tab,
                                                                      const __grid_constant__ SweepTabs T,
                                                                      const LensArgs L0, const int interval,
                                                                      const int service) {
  using M = Mol32<false, false>;
  extern __shared__ float4 s_dyn[];
  __shared__ BlockTally S;
  __shared__ unsigned s_wcount[kT / 32];
  __shared__ int s_left;
  int max_int = 0;
  for (int t = 0; t < n_tab; ++t) max_int = max(max_int, T.n_int[t]);
  SwapSlot* s_swap = reinterpret_cast<SwapSlot*>(s_dyn + (kStaged ? max_int : 0));
  tally_init(S);
  // first table: the one whose share of the queued molecules holds this CTA's
  unsigned total = 0;
  for (int t = 0; t < n_tab; ++t) total += *(volatile unsigned*)Qs.q[t].count;
  const float pos = (float(blockIdx.x) + 0.5f) / float(gridDim.x) * float(total);
  int t0 = n_tab - 1;
  for (unsigned cum = 0, t = 0; t < unsigned(n_tab); ++t) {
    cum += *(volatile unsigned*)Qs.q[t].count;
    if (pos < float(cum)) {
      t0 = int(t);
      break;
    }
  }
  PersistAcc acc;
  for (int k = 0; k < n_tab; ++k) {
    const int t = (t0 + k) % n_tab;
    const Queue& Q = Qs.q[t];
    __syncthreads();  // the previous table's last reads of s_dyn / s_left are done
    if (threadIdx.x == 0) s_left = *(volatile unsigned*)Q.head < *(volatile unsigned*)Q.count;
    __syncthreads();
    if (!s_left) continue;
    if (kStaged)
      for (int j = threadIdx.x; j < T.n_int[t]; j += blockDim.x) s_dyn[j] = __ldg(T.q[t] + j);
    __syncthreads();
    LensArgs L = L0;
    L.q = T.q[t];
    L.s0 = T.s0[t];
    L.n_int = T.n_int[t];
    L.n_smem = kStaged ? T.n_int[t] : 0;
    // no interleaved first entries: each CTA takes from its table's queue in order
    persist_pass<M, false, F, kStaged, kModeSweep, kT>(P, R, li, Q, Q, L, T.order[t], interval, service, 0u, s_dyn,
                                                  s_swap, s_wcount, S, acc, T.done[t], T.done_cap[t]);
  }
  persist_flush(S, R, P.n_labels, acc);
}

// ---------------------------------------------------------------------------
// Ring recording, appended so that no write lands on a newer one and the
// rows and index entries of a run are taken in one order: records are
// numbered by slot (molecules lost inside the recorded lens: their record
// slot, rec_n > 0 staged records; then the molecules stopped by its entrance
// test: one record each), k_ring_count sums each block's contiguous range of
// records, k_ring_scan turns the sums into each block's first row and index
// entry after the ring's heads (and advances the heads), k_ring_reserve gives
// every record its rows and entry in slot order, and k_ring_write reads the
// final heads and writes only what lies within the last capacity_rows rows /
// capacity_molecules entries, where positions are distinct.  Because rows and
// entries follow one order, the latest index entries hold the latest rows.
constexpr int kRingBlocks = 512, kRingThreads = 256;

__device__ __forceinline__ int ring_record_rows(const RunDev& R, unsigned s, unsigned n_slots) {
  return s < n_slots ? R.rec_n[s] : 1;
}

// Block-wide inclusive scan of (a, b) over the threads of a kRingThreads block.
__device__ __forceinline__ void ring_block_scan(unsigned long long& a, unsigned long long& b,
                                                unsigned long long* s_a, unsigned long long* s_b) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long va = __shfl_up_sync(kFull, a, o), vb = __shfl_up_sync(kFull, b, o);
    if (lane >= o) {
      a += va;
      b += vb;
    }
  }
  if (lane == 31) {
    s_a[warp] = a;
    s_b[warp] = b;
  }
  __syncthreads();
  unsigned long long pa = 0, pb = 0;
  for (int w = 0; w < warp; ++w) {
    pa += s_a[w];
    pb += s_b[w];
  }
  a += pa;
  b += pb;
  __syncthreads();
}

static __global__ void __launch_bounds__(kRingThreads) k_ring_count(const RunDev R, unsigned n_slots,
                                                                    unsigned long long* part) {
  __shared__ unsigned long long s_a[kRingThreads / 32], s_b[kRingThreads / 32];
  unsigned lo, hi;
  order_range(n_slots + *R.ent_count, lo, hi);
  unsigned long long rows = 0, recs = 0;
  for (unsigned s = lo + threadIdx.x; s < hi; s += blockDim.x) {
    const int k = ring_record_rows(R, s, n_slots);
    if (k > 0) {
      rows += (unsigned long long)k;
      ++recs;
    }
  }
  ring_block_scan(rows, recs, s_a, s_b);
  if (threadIdx.x == blockDim.x - 1) {
    part[2 * blockIdx.x] = rows;
    part[2 * blockIdx.x + 1] = recs;
  }
}

static __global__ void __launch_bounds__(kRingBlocks) k_ring_scan(const RunDev R, unsigned long long* part) {
  __shared__ unsigned long long s_a[kRingBlocks / 32], s_b[kRingBlocks / 32];
  const ctraj_ring& G = R.ring;
  const int t = threadIdx.x;
  const unsigned long long own_r = part[2 * t], own_m = part[2 * t + 1];
  unsigned long long r = own_r, m = own_m;
  // inclusive scan over the kRingBlocks blocks (warp scans, then the warps' totals)
  const int lane = t & 31, warp = t >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const unsigned long long vr = __shfl_up_sync(kFull, r, o), vm = __shfl_up_sync(kFull, m, o);
    if (lane >= o) {
      r += vr;
      m += vm;
    }
  }
  if (lane == 31) {
    s_a[warp] = r;
    s_b[warp] = m;
  }
  __syncthreads();
  unsigned long long pr = 0, pm = 0;
  for (int w = 0; w < warp; ++w) {
    pr += s_a[w];
    pm += s_b[w];
  }
  r += pr;
  m += pm;
  const unsigned long long h0 = G.heads[0], h1 = G.heads[1];
  __syncthreads();  // every thread has read the heads before the last one moves them
  part[2 * t] = h0 + r - own_r;  // the block's first row and index entry
  part[2 * t + 1] = h1 + m - own_m;
  if (t == kRingBlocks - 1) {
    G.heads[0] = h0 + r;
    G.heads[1] = h1 + m;
  }
}

static __global__ void __launch_bounds__(kRingThreads) k_ring_reserve(const RunDev R, unsigned n_slots,
                                                                      const unsigned long long* part) {
  __shared__ unsigned long long s_a[kRingThreads / 32], s_b[kRingThreads / 32];
  unsigned lo, hi;
  order_range(n_slots + *R.ent_count, lo, hi);
  unsigned long long rbase = part[2 * blockIdx.x], mbase = part[2 * blockIdx.x + 1];
  for (unsigned c0 = lo; c0 < hi; c0 += blockDim.x) {  // block-uniform
    const unsigned s = c0 + threadIdx.x;
    const int k = s < hi ? ring_record_rows(R, s, n_slots) : 0;
    const bool take = k > 0;
    unsigned long long rows = take ? (unsigned long long)k : 0, recs = take ? 1 : 0;
    ring_block_scan(rows, recs, s_a, s_b);  // inclusive
    if (take) {
      const unsigned long long r0 = rbase + rows - (unsigned long long)k, m0 = mbase + recs - 1;
      if (s < n_slots) {
        R.rec_r0[s] = r0;
        R.rec_m0[s] = m0;
      } else {
        R.ent_r0[s - n_slots] = r0;
        R.ent_m0[s - n_slots] = m0;
      }
    }
    // the chunk's totals: the last thread's inclusive sums
    if (threadIdx.x == blockDim.x - 1) {
      s_a[0] = rows;
      s_b[0] = recs;
    }
    __syncthreads();
    rbase += s_a[0];
    mbase += s_b[0];
    __syncthreads();
  }
}

// z and t of a record after k RK4 steps are z0 + k dz and t0 + k dt with the
// molecule's own step (electrostatic_lens.py:87-88), in double, as the
// trajectory rows of the replay kernel have them.  A molecule stopped by the
// entrance test is re-walked from its initial conditions to the entrance.
template <class M>
__global__ void __launch_bounds__(256) k_ring_write(const __grid_constant__ Plan P, const RunDev R,
                                                    unsigned n_slots) {
  const ctraj_element& e = P.el[R.rec_lens];
  const ctraj_ring& G = R.ring;
  const unsigned n_ent = *R.ent_count;
  const unsigned long long hr = G.heads[0], hm = G.heads[1];
  const unsigned long long cr = (unsigned long long)G.capacity_rows, cm = (unsigned long long)G.capacity_molecules;
  const unsigned stride = gridDim.x * blockDim.x;
  for (unsigned s = blockIdx.x * blockDim.x + threadIdx.x; s < n_slots + n_ent; s += stride) {
    if (s < n_slots) {
      const int n_rec = R.rec_n[s];
      if (n_rec <= 0) continue;
      const unsigned long long r0 = R.rec_r0[s], m0 = R.rec_m0[s];
      const float vz = R.rec_vz[s];
      LensStep st;
      lens_setup(e, double(vz), st);
      const int last = R.rec_last[s];
      const double t0 = double(R.rec_t0[s]);
      for (int j = 0; j < n_rec; ++j) {
        if (r0 + j + cr < hr) continue;  // overwritten by a newer record
        const int k = j == n_rec - 1 ? last : j * R.rec_stride;
        const float4 a = R.rec[size_t(s) * R.rec_max + j];
        ring_row(G, r0 + j, a.x, a.y, float(e.z0 + double(k) * st.dz), a.z, a.w, vz,
                 float(t0 + double(k) * st.dt), float(k));
      }
      if (m0 + cm >= hm) ring_entry(G, m0, int64_t(R.offset) + R.rec_id[s], r0, n_rec, e.label_inside);
    } else {
      const unsigned k = s - n_slots;
      const unsigned long long r0 = R.ent_r0[k], m0 = R.ent_m0[k];
      const int32_t id = R.ent_id[k];
      M m;
      m.init(P, R, id);
      int lens_at = -1;
      const int label = walk(m, P, 0, &lens_at);
      if (r0 + cr >= hr) ring_row(G, r0, m.x, m.y, float(e.z0), m.vx, m.vy, m.vz, m.t, 0.0f);
      if (m0 + cm >= hm) ring_entry(G, m0, int64_t(R.offset) + id, r0, 1, label);
    }
  }
}

// ---------------------------------------------------------------------------
// Replay of selected molecules with row recording (one thread per molecule).
template <class M>
__device__ __forceinline__ bool step_any(M& m, const Plan& P, int li, const float dt, const float hdt,
                                         const float c2, const float dt6, const float dt26,
                                         unsigned& flags) {
  const LensArgs L = lens_args(P, li, false);  // no shared-memory copy: tables from global memory
  switch (P.lf[li].force) {
    case kForceStark2:
      return m.template lens_step<kForceStark2, false>(L, dt, hdt, c2, dt6, dt26, nullptr, flags);
    case kForceStark2Lin:
      return m.template lens_step<kForceStark2Lin, false>(L, dt, hdt, c2, dt6, dt26, nullptr, flags);
    case kForceStark1:
      return m.template lens_step<kForceStark1, false>(L, dt, hdt, c2, dt6, dt26, nullptr, flags);
    default:
      return m.template lens_step<kForceRadial, false>(L, dt, hdt, c2, dt6, dt26, nullptr, flags) ||
             (flags & 2u);
  }
}

// The whole path of one molecule with every trajectory row sent to m.sink.
template <class M, bool k64>
__device__ void replay(M& m, const Plan& P) {
  int from = 0;
  for (;;) {
    int lens_at = -1;
    const int label = walk(m, P, from, &lens_at);
    if (label != kQueued) break;
    const ctraj_element& e = P.el[lens_at];
    LensStep st;
    if (!lens_setup(e, m.vel_z(), st)) break;
    m.lens_begin(P, lens_at, st);
    const float dt = float(st.dt), hdt = 0.5f * dt;
    const float c2 = e.scheme == CTRAJ_RK4_CLASSIC ? hdt : dt;
    const float dt6 = dt * (1.0f / 6.0f), dt26 = float(st.dt * st.dt / 6.0);
    bool lost = false;
    unsigned flags = 0;
    while (st.n_done < st.n_total) {
      if constexpr (k64) {
        int rg = 0, er = 0;
        lost = m.lens_step(P, lens_at, st, rg, er);
      } else {
        lost = step_any(m, P, lens_at, dt, hdt, c2, dt6, dt26, flags);
      }
      ++st.n_done;
      m.lens_row(P, lens_at, st);
      if (lost) break;
    }
    m.lens_end(P, lens_at, st, lost);
    if (lost) break;
    from = lens_at + 1;
  }
  m.flush_last();
}

template <class M, bool k64>
__global__ void __launch_bounds__(128) k_record(const __grid_constant__ Plan P, const RunDev R,
                                                const int64_t* ids, int64_t n_ids, int stride,
                                                int max_rows, double* rows_out, int32_t* count_out,
                                                unsigned* overflow) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n_ids) return;
  RowSink sink{rows_out + size_t(k) * size_t(max_rows) * 10, max_rows, stride, 0, 0, false};
  M m;
  m.sink = &sink;
  m.init(P, R, ids[k]);
  replay<M, k64>(m, P);
  count_out[k] = sink.written;
  if (sink.written > max_rows) atomicAdd(overflow, 1u);
}

// z-plane post-processing (post_processing.py:20-140): replay each molecule and
// return its position and velocity at the plane z = zp, taken from the row at
// zp or advanced from the row before it by x + v dt + a dt^2 / 2, v + a dt with
// dt = (zp - z) / vz (take_timestep, :9-17), in double.  out: (n_ids, 8) =
// x, y, z, vx, vy, vz, status (0: the molecule ends before the plane, 1:
// advanced, 2: a row lies on the plane), 0.
template <class M, bool k64>
__global__ void __launch_bounds__(128) k_plane(const __grid_constant__ Plan P, const RunDev R, const int64_t* ids,
                                               int64_t n_ids, double zp, double* out) {
  const int64_t k = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (k >= n_ids) return;
  RowSink sink{nullptr, 0, 1, 0, 0, false};
  sink.plane = true;
  sink.zp = zp;
  M m;
  m.sink = &sink;
  m.init(P, R, ids[k]);
  replay<M, k64>(m, P);
  double* o = out + size_t(k) * 8;
  for (int c = 0; c < 8; ++c) o[c] = c < 6 ? nan("") : 0.0;
  if (sink.written == 0 || sink.last[2] < zp) return;  // molecule.x()[2] < z: skipped
  if (sink.pexact) {
    for (int c = 0; c < 6; ++c) o[c] = sink.exact[c];
    o[6] = 2.0;
    return;
  }
  const double* h = sink.pcross == 3 ? sink.last : sink.hit;
  const double dt = (zp - h[2]) / h[5];
  const double dt2 = dmul(dt, dt);
  for (int c = 0; c < 3; ++c) {
    o[c] = dadd(dadd(h[c], dmul(h[3 + c], dt)), dmul(h[6 + c], dt2) / 2.0);
    o[3 + c] = dadd(h[3 + c], dmul(h[6 + c], dt));
  }
  o[6] = 1.0;
}

}  // namespace ctraj
