// Launch-time description of a beamline, shared by every kernel.
//
// The host builds one Plan per run from the ctraj_element table (kept
// verbatim for the FP64 path) plus FP32 constants precomputed in double on the
// host (plane-to-plane gaps, squared radii, table scale factors), and passes it
// by value as a __grid_constant__ kernel parameter: every thread of a warp
// reads the same element at the same time, so the constant cache broadcasts.
#pragma once
#include <cstdint>

#include "ctraj.h"
#include "philox.cuh"

namespace ctraj {

enum : int {
  kForceStark2 = 0,  // W(E) table, |E| = alpha r^2
  kForceStark1 = 1,  // W(E) table, |E| = alpha r
  kForceRadial = 2,  // a(r) linear table
  // W(E) table, |E| = alpha r^2, whose derivative is tabulated as linear
  // pieces on quarter intervals (float2 (w, dw) entries, two per float4;
  // n_int counts the float4): chosen by the host when that is accurate and
  // the table covers the bore
  kForceStark2Lin = 3,
};

// FP32 constants of one element.
struct ElemF {
  float gap;   // (float)(z0 - z1 of the previous element); flight into this element
  float len;   // (float)(z1 - z0)
  float c[4];  // circle: (d/2)^2; rect: x1, x2, y1, y2; plates: x1, x2; lens: (d/2)^2;
               // honeycomb: R sqrt(3)/2, R, 1 / row pitch, 1 / cell pitch
};

// FP32 constants of one lens (indexed by element).
struct LensF {
  const float4* q;  // per interval: stark (q0, q1, q2, 0) scaled by -kappa; stark2lin two float4
                    // of two pieces (w, dw, w, dw) scaled by -kappa; radial (y_j, y_{j+1}-y_j, 0, 0)
  float beta;       // table coordinate s = beta * r^n - s0 (stark; stark2lin in quarter intervals)
                    // or r * beta (radial, beta = 1/h)
  float s0;
  float r_max;      // radial: last knot; lookups above it are errors
  int n_int;        // float4 entries of the table (intervals; stark2lin 2 per interval)
  int n_smem;       // leading intervals staged in shared memory
  int force;        // kForce*
  int cols;         // honeycomb: q = cell centres (x, y, 0, 0), n_int = cells, cols = cells per row
  int outward;      // stark: w >= 0 over the whole table, the force points away from the axis
};

// The FP32 constants of the one lens a k_lens_chunk launch integrates, passed
// as their own kernel parameter so every use is a fixed-offset constant-bank
// operand (the Plan's per-element arrays need an indexed load per use).
struct LensArgs {
  const float4* q;
  float beta, s0, r_max;
  int n_int, n_smem;
  float g;
  float bore2;  // (d/2)^2
  float bore;   // d/2
  int classic;
};

// FP64 view of a force table (device pointers).
struct TableD {
  const double* knots;
  const double* coef;    // (n-1) x 4
  const double* values;  // n
  double x0, h;          // first knot, uniform spacing
  int n;
  int kind;
};

struct Plan {
  int n_el;
  int n_labels;
  int first_lens;  // index of the first lens element, n_el if none
  int pad;
  double g;
  float gf;
  float pad2;
  ctraj_element el[CTRAJ_MAX_ELEMENTS];
  ElemF ef[CTRAJ_MAX_ELEMENTS];
  LensF lf[CTRAJ_MAX_ELEMENTS];
  TableD td[CTRAJ_MAX_TABLES];
};

// LensArgs of lens element li; staged = false reads the whole table from
// global memory (no shared-memory copy).
__host__ __device__ inline LensArgs lens_args(const Plan& P, int li, bool staged) {
  const LensF& f = P.lf[li];
  LensArgs a;
  a.q = f.q;
  a.beta = f.beta;
  a.s0 = f.s0;
  a.r_max = f.r_max;
  a.n_int = f.n_int;
  a.n_smem = staged ? f.n_smem : 0;
  a.g = P.gf;
  a.bore2 = P.ef[li].c[0];
  a.bore = P.ef[li].c[1];
  a.classic = P.el[li].scheme == CTRAJ_RK4_CLASSIC;
  return a;
}

// Per-run device pointers and scalars.
struct RunDev {
  int64_t n;
  uint64_t seed;
  PhiloxKey key;  // round keys of seed
  uint64_t offset;
  int ic_mode;
  int pad;
  const double* ics;  // (6, n) when injected
  ctraj_distribution xd, vd;
  float gap0f;         // FP32 first flight for drawn ICs: (float)(el[0].z0 - xd.z)
  float pad3;
  int32_t* out_label;
  double* out_final;   // (10, n)
  int32_t* out_rows;
  double* out_margin;
  unsigned long long* counts;  // n_labels + 1
  unsigned long long* stats;   // kStat*
  // batched sweep: molecule i belongs to configuration c with
  // cfg_start[c] <= i < cfg_start[c + 1]; each configuration has its own
  // lens voltage (table coordinate scale beta and force scale kappa) and
  // Stark table; counts are kept per configuration in cfg_counts.
  int n_cfg;
  int pad4;
  const int64_t* cfg_start;   // n_cfg + 1
  const float* cfg_beta;      // n_cfg
  const float* cfg_kappa;     // n_cfg
  const int32_t* cfg_table;   // n_cfg: which lens queue / table
  unsigned long long* cfg_counts;  // n_cfg x (n_labels + 1)
  // grouped batch (ctraj_run_batch): the runs of a group share one lens
  // queue; a molecule carries its run's index in the group (Queue::cfg, set
  // by the run's front launch from run_tag), its counts go to cfg_counts and
  // its stats to cfg_stats (runs x kStatCount), both indexed by that run.
  int run_tag;
  int pad5;
  unsigned long long* cfg_stats;
  // ring recording (ctraj_run_ring): the molecules reaching lens rec_lens get
  // a record slot (their queue position at the front, carried in Queue::cfg);
  // (x, y, vx, vy) is staged every rec_stride RK4 steps, and the molecules
  // lost on the lens are appended to the ring by k_ring_gather.
  int rec_lens;               // -1: off
  int rec_stride;
  int rec_max;                // staged records per slot
  int rec_entrance_label;     // counter slot of the recorded lens's entrance test
  float4* rec;                // (slots, rec_max)
  int32_t* rec_n;             // per slot: records staged if lost inside the lens, else 0
  int32_t* rec_last;          // per slot: RK4 steps done when lost
  int32_t* rec_id;            // per slot: molecule index
  float* rec_t0;              // per slot: time at the lens entrance
  float* rec_vz;
  unsigned long long* rec_r0; // per slot: first ring row and index entry taken
  unsigned long long* rec_m0;
  int32_t* ent_id;            // molecules stopped by the entrance test (listed by k_front)
  unsigned* ent_count;
  unsigned long long* ent_r0;
  unsigned long long* ent_m0;
  ctraj_ring ring;
};

enum : int {
  kStatSteps = 0,
  kStatLensSteps = 1,
  kStatEdgeBand = 2,
  kStatTableRange = 3,
  kStatBadSteps = 4,
  kStatRangeError = 5,
  kStatMaxSteps = 6,  // grouped batch: largest step bound queued at a lens (atomicMax, not a sum)
  kStatCount = 8,
};

// Kernel modes: a plain run, a batched sweep (molecules carry their lens
// configuration), ring recording (molecules carry their record slot), a
// grouped batch (molecules carry their run).
enum : int { kModePlain = 0, kModeSweep = 1, kModeRing = 2, kModeBatch = 3 };

// Molecules inside a lens between two chunks of RK4 steps (SoA, capacity n):
// the state, the carried rounding errors of the FP32 integration, and the
// per-molecule step parameters computed once at the lens entrance.  FP32
// queues use the float arrays, FP64 queues the double ones.
struct Queue {
  float *x, *y, *vx, *vy, *vz, *t;     // t: time at the lens entrance
  float *cx, *cy, *cvx, *cvy;
  float* snap;                          // exit-snap time
  double *dx, *dy, *dz, *dvx, *dvy, *dvz, *dt;
  double* lens_dt;                      // dz / vz
  double* margin;
  int32_t* rows;
  int32_t* id;
  int32_t* n_done;
  int32_t* n_total;
  int32_t* cfg;         // configuration (batched sweeps) or record slot (ring recording)
  unsigned int* count;      // entries written
  unsigned int* max_steps;  // largest n_total - n_done written (sizes the chunk loop)
  unsigned int* head;       // entries taken by the warps of the kernel reading the queue
};

// Queue control words: count, max_steps, head, (unused) -- 16 bytes per queue.
constexpr int kCtlWords = 4;

// Batched sweeps: the lens-entrance queue of each Stark table.
struct SweepQueues {
  Queue q[CTRAJ_MAX_TABLES];
};

constexpr int kLabelDetected = -1;  // counts[n_labels]
constexpr int kQueued = -2;         // waiting at a lens entrance
constexpr int kNone = -3;           // no tally (inactive lane)
constexpr float kEdgeBand = 1e-6f;  // molecules nearer than this to an edge are reported

}  // namespace ctraj
