// Host-side internals of libctraj.so shared by its translation units: error
// reporting, device buffers, the context (struct ctraj_context of ctraj.h),
// the beamline plan builders, and the launchers of the kernel families, each
// compiled in translation units of their own (k_front.cu, k_chunk.cu,
// k_persist*.cu) and reached through function pointers -- a kernel launched
// through its host function pointer finds its own module's registration, so
// no device code is linked across units.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "ctraj.h"
#include "plan.cuh"

namespace ctraj {

// The message of the last failing call on this thread (ctraj_last_error).
extern thread_local std::string g_error;

// Records a message for ctraj_last_error and returns code.
int fail(int code, const char* fmt, ...);

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


}  // namespace ctraj

// One context (ctraj_create): its device, stream, beamline, tables, tuning
// and work buffers.
struct ctraj_context {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::vector<ctraj_element> elements;
  int n_labels = 0;
  bool have_beamline = false;
  ctraj::HostTable tables[CTRAJ_MAX_TABLES];
  ctraj::DevBuf lens_tables;           // FP32 lens tables, one region per lens element
  bool lens_tables_dirty = true;
  std::vector<size_t> lens_offset;
  std::vector<int> lens_n_int, lens_n_smem;
  std::vector<int> lens_outward;     // per lens: its FP32 force points away from the axis everywhere
  ctraj::DevBuf queue[3];              // lens queues: current chunk, continuation, next lens
  ctraj::DevBuf qctl;                  // queue counters (2 x unsigned per queue) + counts + stats
  ctraj::DevBuf ics;
  ctraj::DevBuf outs;
  ctraj::DevBuf rec_rows, rec_ids, rec_count;
  unsigned* host_max = nullptr; // pinned: largest remaining lens step count of a queue
  unsigned* host_lens = nullptr; // pinned: per element, its lens queue's largest step bound (async pass)
  bool lens_async = false;      // the last run's lens passes were enqueued without a sync
  ctraj::DevBuf chunk_ctl;             // (count, max_steps) of the queue each lens chunk writes
  ctraj::DevBuf rec_stage;             // ring recording: staged records of the recorded lens
  ctraj::DevBuf ring_ent;              // ring recording: molecules stopped by the entrance test
  ctraj::DevBuf lens_order;            // persistent lens pass: bucket counts | entrant order
  ctraj::DevBuf lens_done;             // persistent lens pass: DoneRec per entrant (deferred ends)
  ctraj::DevBuf ring_part;             // ring recording: per-block row / entry sums and bases
  ctraj::DevBuf sweep_order;           // persistent sweep: per table bucket counts | entrant order
  ctraj::DevBuf sweep_done;            // persistent sweep: per table DoneRec records (deferred ends)
  int chunk = 64;               // RK4 steps of the first lens chunk (compaction interval)
  int chunk_growth = 200;       // percent: each chunk's length relative to the previous
  int chunk_max = 1024;         // longest chunk
  int front_waves = 4;          // k_front grid in units of resident CTAs
  int lens_mode = CTRAJ_LENS_PERSISTENT;  // FP32 lens pass
  int lens_interval = 256;      // persistent mode: steps between CTA compactions
  int lens_service = 64;        // persistent mode: steps between a warp's refills (kPersistService)
  int front_threads = 256;      // k_front block size
  int batch_group = 4;          // ctraj_run_batch: runs sharing one lens pass
  int lens_threads = 512;       // persistent FP32 lens pass: molecule lanes per CTA
  int lens_molecules = 1;       // persistent FP32 lens pass: molecules per thread
  int batch_lens_threads = 1024;  // lens_threads of a batch group's shared lens passes
  unsigned run_max_steps = 0;   // largest lens queue step bound of the last run
  bool timing = false;
  // before front, after front, before the first lens chunk, after the last one
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  // bumped by every call that changes what a captured sweep graph depends on
  uint64_t generation = 0;
  // batched sweeps (ctraj_run_sweep), set up on first use
  ctraj::DevBuf sweep_tables;          // unscaled FP32 Stark tables, one region per table used
  ctraj::DevBuf sweep_cfg;             // per-configuration arrays and counts
  ctraj::DevBuf sweep_ctl;             // queue counters, chunk counters, totals, stats
  ctraj::DevBuf sweep_queue[2 * CTRAJ_MAX_TABLES];
  // soft transmission (ctraj_soft_transmission)
  ctraj::DevBuf soft_table, soft_queue, soft_ckpt, soft_ctl, soft_contrib, soft_seg, soft_post;
  // what soft_table holds: built from table soft_table_id at generation
  // soft_table_gen in elements of soft_table_size bytes, scaled by soft_table_f
  uint64_t soft_table_gen = ~uint64_t(0);
  int soft_table_id = -1, soft_table_size = 0;
  double soft_table_f = 1.0;
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
  ctraj::DevBuf l2_flush;              // scratch written before each run of a batch
  cudaEvent_t batch_ev = nullptr;
  // grouped batches: per-run counts and stats (device and pinned host), the
  // host initial conditions of a group's runs
  ctraj::DevBuf group_ctl;
  unsigned long long* group_host = nullptr;
  size_t group_host_words = 0;
  ctraj::DevBuf group_ics;
};

namespace ctraj {

inline size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

constexpr int kMaxStagedIntervals = 6144;  // 96 KiB of float4 per CTA
// a kForceStark2Lin table (two float4 of pieces per knot interval) is staged
// up to 128 KiB: with the persistent pass's 40 KiB of swap slots one CTA per SM
constexpr int kMaxStagedLinear = 8192;
constexpr int kMaxChunks = 16384;          // lens chunks per lens (CTRAJ_MAX_LENS_STEPS / 1024 < this)

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

// Queue layout inside one buffer of capacity cap (SoA, each array 256-byte
// aligned so a warp's 32 consecutive entries are whole 128-byte lines).
// Returns the bytes used; with b == nullptr only sizes the layout.
size_t layout_queue(const DevBuf* b, size_t cap, int precision, unsigned* ctl, Queue* q, bool with_cfg = false);
size_t queue_bytes(size_t cap, int precision, bool with_cfg = false);
bool stark_linear(int kind, int n_knots, const double* knots, const double* coef, const ctraj_element& e);
float4 stark_pieces(double a, double b, double c, int half);
int lens_force_kind(const ctraj_context* c, const ctraj_element& e);
int build_lens_tables(ctraj_context* c);
void honeycomb_constants(const ctraj_element& e, ElemF& f);
int check_honeycomb(const ctraj_element& e, int i, int kind, int n);
int build_plan(ctraj_context* c, const ctraj_run_args* a, Plan& P);
int check_beamline(const ctraj_context* c);
int validate_run(const ctraj_context* c, const ctraj_run_args* a);
int prepare(ctraj_context* c, const ctraj_run_args* a, Plan& P, RunDev& R);

template <class KernelT>
int blocks_per_sm(KernelT k, int threads, size_t smem) {
  int b = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k, threads, smem) != cudaSuccess || b < 1) b = 1;
  return b;
}

// ---- kernel families (defined in their own translation units) --------------

// k_front over n molecules into queue Q (k_front.cu): precision 32 or 64,
// per-molecule outputs or not, kMode* (plain, ring recording, grouped batch);
// threads per block, a grid of `waves` x resident CTAs (or fewer), the lens
// entrants staged in dynamic shared memory.
int launch_front(const Plan& P, const RunDev& R, const Queue& Q, int64_t n, int precision, bool out, int mode,
                 int threads, int sms, int waves, cudaStream_t s);

// The chunked lens kernel (k_chunk.cu): FP32 specialised on the force law
// (kForce*), staged table or not, ring recording; FP64 evaluates the
// reference's force code for every table kind.  sweep_lens_kernel: the
// chunked pass of a batched sweep.
using LensKernel = void (*)(const Plan, const RunDev, const int, const Queue, const Queue, const Queue, const int,
                            const LensArgs);
LensKernel lens_kernel(bool k64, bool out, bool ring, int force, bool staged);
LensKernel sweep_lens_kernel(int force, bool staged);

// The persistent FP32 lens kernel (k_persist.cu) for force law `force`, mode
// kMode* (plain, ring, batch), staged table or not; lanes: molecules per CTA
// (tuning lens_threads), mpt: molecules per thread (tuning lens_molecules).
// *threads and *used_mpt receive the CTA size and molecules per thread of the
// kernel returned.  512, 768 or 1024 lanes at one molecule per thread, and
// for the hexapole Stark forms also at two, are compiled for the staged-table
// plain and batch passes without per-molecule outputs (the throughput path);
// every other pass and setting runs 512 threads x 1.
struct DoneRec;  // kernels.cuh: a molecule's state after its last step, for k_lens_finish
using PersistKernel = void (*)(const Plan, const RunDev, const int, const Queue, const Queue, const LensArgs,
                               const unsigned*, const int, const int, DoneRec*);
PersistKernel persist_kernel(bool out, int force, int mode, bool staged, int lanes, int mpt, int* threads,
                             int* used_mpt);
template <int F>  // one force law's configurations (k_persist_<law>.cu)
PersistKernel persist_kernel_for(bool out, int mode, bool staged, int lanes, int mpt, int* threads, int* used_mpt);

// k_lens_finish for a plain, batch or sweep pass (k_persist.cu).
using FinishKernel = void (*)(const Plan, const RunDev, const int, const Queue, const Queue, const DoneRec*,
                              const unsigned);
FinishKernel finish_kernel(int mode);
constexpr size_t kDoneRecBytes = 64;

// The persistent FP32 lens pass of lens element i over queue Qin (ctraj.cu):
// the entrants ordered longest first into `order_buf` (kOrderBuckets + the
// queue's entries), then one k_lens_persist launch, one CTA per SM.  With
// `done` (kDoneRecBytes per queue entry; plain or batch passes without
// per-molecule outputs) the molecules' ends are deferred to one k_lens_finish
// launch after the pass.
int enqueue_persistent(bool out, int mode, const Plan& P, const RunDev& R, int i, const Queue& Qin,
                       const Queue& Qnext, unsigned* order_buf, int sms, int interval, int service, cudaStream_t s,
                       int* launches, int lanes, int mpt, DoneRec* done = nullptr);

}  // namespace ctraj
