/*
 * ctraj.h -- C ABI of the GB300 trajectory engine (libctraj.so).
 *
 * The engine propagates molecules through a z-sorted beamline the way the
 * reference package ``trajectories`` does in pure Python:
 *
 *   TrajectorySimulator.run_simulation     src/trajectories/trajectory_simulator.py:34-103
 *   Beamline.propagate_through             src/trajectories/beamline.py:20-38
 *   Molecule.x/v/update_trajectory         src/trajectories/molecule.py:26-68
 *   CircularAperture.propagate_through     src/trajectories/beamline_elements/apertures.py:92-115
 *   RectangularAperture.propagate_through  src/trajectories/beamline_elements/apertures.py:165-189
 *   FieldPlates.propagate_through          src/trajectories/beamline_elements/apertures.py:227-270
 *   ElectrostaticLens.propagate_through    src/trajectories/beamline_elements/electrostatic_lens.py:48-118
 *   ElectrostaticLens.lens_acceleration    src/trajectories/beamline_elements/electrostatic_lens.py:168-227
 *   Distribution.draw (known subclasses)   src/trajectories/distributions.py:40-41,69-76,112-119,155-162
 *   Counter.increment_counter              src/trajectories/trajectory_simulator.py:117-124
 *
 * The reference has no foreign-function interface of its own (it is ~2 kLoC of
 * Python); every entry point below replaces the Python function cited beside
 * it, and the Python package shipped with this library (ctraj._abi) binds them
 * through ctypes.
 *
 * Conventions: every function returns an int status (CTRAJ_OK == 0, negative
 * on error) and never throws.  ctraj_last_error() returns a message for the
 * last failing call on the calling thread.  Host pointers are owned by the
 * caller; device memory is owned by the context.  A context is bound to one
 * CUDA device and one stream; calls on one context must not overlap in time.
 */
#ifndef CTRAJ_H_
#define CTRAJ_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CTRAJ_ABI_VERSION 2

/* ---- status codes -------------------------------------------------------- */
enum {
  CTRAJ_OK = 0,
  CTRAJ_EINVAL = -1,    /* bad argument (unknown element type, n < 0, ...)              */
  CTRAJ_ECUDA = -2,     /* CUDA runtime error                                            */
  CTRAJ_ENOMEM = -3,    /* device allocation failed                                      */
  CTRAJ_ERANGE = -4,    /* bounded force table looked up outside its knots; the reference
                           raises ValueError from interp1d there (electrostatic_lens.py:217) */
  CTRAJ_ESTEPS = -5,    /* lens step count rint(L/dz) not finite or above CTRAJ_MAX_LENS_STEPS;
                           the reference raises OverflowError/MemoryError there (:87)     */
  CTRAJ_EOVERFLOW = -6, /* trajectory record buffer too small                            */
  CTRAJ_ESTATE = -7,    /* call order violated (run before set_beamline, ...)            */
};

#define CTRAJ_MAX_ELEMENTS 64
#define CTRAJ_MAX_LABELS 64
#define CTRAJ_MAX_TABLES 8
#define CTRAJ_MAX_LENS_STEPS 10000000LL

/* ---- beamline elements ---------------------------------------------------- */
enum {
  CTRAJ_CIRCULAR_APERTURE = 1,    /* apertures.py:84-122  */
  CTRAJ_RECTANGULAR_APERTURE = 2, /* apertures.py:147-196 */
  CTRAJ_FIELD_PLATES = 3,         /* apertures.py:213-277 */
  CTRAJ_ELECTROSTATIC_LENS = 4,   /* electrostatic_lens.py:23-125 */
  CTRAJ_HONEYCOMB = 5,            /* meshes.py:26-178 */
};

enum { CTRAJ_STEP_DZ = 0, CTRAJ_STEP_DT = 1 };           /* lens step mode  */
enum { CTRAJ_RK4_REFERENCE = 0, CTRAJ_RK4_CLASSIC = 1 }; /* lens RK4 scheme */

/*
 * One beamline element, in the order the molecules meet them (sorted by z0,
 * beamline.py:40-45).  Geometry is passed exactly as the reference computes it
 * in __post_init__ (z1 = z0 + L, x1 = x0 - w/2, ...) so both sides compare the
 * same doubles.
 *
 *   p[] per type
 *   circular aperture : p[0] = d (diameter)
 *   rectangular       : p[0] = x1, p[1] = x2, p[2] = y1, p[3] = y2 (w spans X, h spans Y)
 *   field plates      : p[0] = x1, p[1] = x2
 *   honeycomb         : p[0] = circumradius of each cell's hexagon (pointy side
 *                       along y, the matplotlib RegularPolygon of meshes.py:71-78);
 *                       table = a CTRAJ_TABLE_MESH with the cell centres of an
 *                       hexalattice grid (rows of p[1] cells, odd rows shifted
 *                       by half a pitch); p[1] = cells per row, p[2] = 1 / row
 *                       pitch in y, p[3] = 1 / cell pitch in x.  p[1..3] only
 *                       place the device's nearest-centre search window (5 x 5
 *                       cells around the estimate, 4 rows at the grid's ends);
 *                       the cell found is the reference's argmin over all
 *                       centres for such a grid.
 *   electrostatic lens: p[0] = d (bore diameter), p[1] = dz, p[2] = dt,
 *                       p[3] = V (electrode voltage), p[4] = R (field radius),
 *                       p[5] = mass (kg), p[6] = alpha with |E| = alpha r^n
 *                       (c V / R^(n+1), computed by the caller so every
 *                       backend sees the same double), p[7] = L
 *
 * label        counter slot credited when a molecule is lost on this element
 *              (for the lens: the "Lens entrance" slot, electrostatic_lens.py:63)
 * label_inside lens only: the "Inside lens" slot (electrostatic_lens.py:117)
 * table        lens: force table id (ctraj_set_force_table); honeycomb: mesh table id
 * step_mode    lens only: CTRAJ_STEP_DZ -> N = rint(L/dz), dt = dz/vz (:87-88);
 *              CTRAJ_STEP_DT -> dz = vz*dt per molecule, then as DZ
 * scheme       lens only: CTRAJ_RK4_REFERENCE reproduces the reference's stage-2
 *              point x + dt*k1 (:97); CTRAJ_RK4_CLASSIC uses x + dt*k1/2
 * field_order  lens + W(E) table only: |E| = c V r^n / R^(n+1), n = 1 (c = 2, the
 *              reference's own field model, :200) or n = 2 (c = 3, hexapole)
 */
typedef struct ctraj_element {
  int32_t type;
  int32_t label;
  int32_t label_inside;
  int32_t table;
  int32_t step_mode;
  int32_t scheme;
  int32_t field_order;
  int32_t reserved;
  double z0, z1, x0, y0;
  double p[8];
} ctraj_element;

/* ---- lens force tables ---------------------------------------------------- */
enum {
  /* Stark energy W(E) as a piecewise cubic on uniform knots in |E| (V/m); the
   * force is -dW/dE * grad|E| / m.  coef is (n_knots-1) x 4 in scipy PPoly
   * order (t^3, t^2, t, 1) per interval, t = E - knots[i].  Lookups beyond the
   * knots extrapolate the boundary piece, as scipy CubicSpline does.          */
  CTRAJ_TABLE_STARK_SPLINE = 1,
  /* Radial acceleration a(r) (m/s^2) linear between uniform knots in r (m),
   * the reference's interp1d table (electrostatic_lens.py:194-209).  Lookups
   * above the last knot are errors (CTRAJ_ERANGE), as interp1d raises.        */
  CTRAJ_TABLE_RADIAL_LINEAR = 2,
  /* Cell centres of a honeycomb mesh: knots = x, values = y (n_knots cells, in
   * the order the nearest-centre search scans them, meshes.py:104-108).       */
  CTRAJ_TABLE_MESH = 3,
};

typedef struct ctraj_force_table {
  int32_t kind;
  int32_t n_knots;
  const double* knots;  /* n_knots; STARK_SPLINE, RADIAL_LINEAR: ascending and
                           uniformly spaced; MESH: cell centre x, any order    */
  const double* coef;   /* STARK_SPLINE: (n_knots - 1) * 4                    */
  const double* values; /* RADIAL_LINEAR, MESH: n_knots                       */
} ctraj_force_table;

/* ---- initial-condition distributions (distributions.py) ------------------- */
enum {
  CTRAJ_DIST_NONE = 0,
  CTRAJ_DIST_GAUSSIAN_POSITION = 1, /* p = {sigmax, sigmay, z}            (:144-162) */
  CTRAJ_DIST_DISC_POSITION = 2,     /* p = {d, z}                         (:101-119) */
  CTRAJ_DIST_GAUSSIAN_VELOCITY = 3, /* p = {vx, sigmax, vy, sigmay, vz, sigmaz} (:55-76) */
};

typedef struct ctraj_distribution {
  int32_t kind;
  int32_t reserved;
  double p[6];
} ctraj_distribution;

enum { CTRAJ_IC_DEVICE_DRAW = 0, CTRAJ_IC_HOST = 1, CTRAJ_IC_DEVICE = 2 };
enum { CTRAJ_OUT_NONE = 0, CTRAJ_OUT_HOST = 1, CTRAJ_OUT_DEVICE = 2 };

/*
 * One propagation run of n molecules (the body of trajectory_simulator.py:52-78
 * for all chunks at once).
 *
 * precision  32: FP32 state, transverse force from the table with z held
 *            relative to element planes; 64: FP64 with the reference's own
 *            operation order (bit-for-bit the reference on ballistic paths).
 * ic_mode    CTRAJ_IC_DEVICE_DRAW: positions from xdist and velocities from
 *            vdist drawn on the device with Philox-4x32-10 keyed by seed,
 *            molecule i using counter (offset + i); CTRAJ_IC_HOST/DEVICE: ics
 *            points to a (6, n) row-major float64 array x, y, z, vx, vy, vz
 *            (the reference's xs / vs stacked, trajectory_simulator.py:57-58).
 * out_*      optional per-molecule results (out_mode says host or device
 *            pointers; NULL entries are skipped): out_label[i] counter slot,
 *            or -1 for "Detected"; out_final (10, n) last trajectory row
 *            x, y, z, vx, vy, vz, ax, ay, az, t; out_rows[i] = len(t) - 1 of
 *            the reference trajectory; out_margin[i] smallest distance to an
 *            edge seen by any hit test along the path (m).
 * counts     host array of n_labels + 1 int64: per-label losses, then the
 *            "Detected" count in counts[n_labels].
 */
typedef struct ctraj_run_args {
  int64_t n;
  int32_t precision;
  int32_t ic_mode;
  const double* ics;
  ctraj_distribution xdist;
  ctraj_distribution vdist;
  uint64_t seed;
  uint64_t offset;
  double g;
  int32_t out_mode;
  int32_t timing;           /* nonzero: time the kernels with CUDA events (stats) */
  int32_t* out_label;
  double* out_final;
  int32_t* out_rows;
  double* out_margin;
  int64_t* counts;
} ctraj_run_args;

typedef struct ctraj_run_stats {
  int64_t molecules;        /* molecules propagated                           */
  int64_t molecule_steps;   /* sum over molecules of len(trajectory.t) - 1    */
  int64_t lens_steps;       /* RK4 steps (subset of molecule_steps)           */
  int64_t edge_band;        /* molecules whose smallest edge distance < 1 um  */
  int64_t table_range;      /* lookups outside a table's knots                */
  int64_t bad_steps;        /* molecules with a non-finite lens step count    */
  int32_t kernels;          /* kernel launches issued by this run             */
  int32_t timed;            /* 1 when the *_ms fields below were measured     */
  float front_ms;           /* CUDA-event time of the ballistic front kernel  */
  float lens_ms;            /* CUDA-event time of all lens kernels            */
  int32_t max_lens_steps;   /* ctraj_run, ctraj_run_batch, ctraj_run_noalloc:
                               upper bound on the RK4 steps of the molecule
                               with the most steps in a lens (rint(L/dz) + 2),
                               the length of the lens pass's critical path; 0
                               from the other entry points                    */
  int32_t linear_tables;    /* ctraj_run, ctraj_run_batch, ctraj_run_noalloc:
                               lens elements whose FP32 run used the 8-byte
                               linear form of their Stark table (the host's
                               accuracy and coverage test passed)             */
} ctraj_run_stats;

/* ---- context -------------------------------------------------------------- */
typedef struct ctraj_context ctraj_context;

int ctraj_version(void);
const char* ctraj_last_error(void);

int ctraj_create(int device, ctraj_context** out);
int ctraj_destroy(ctraj_context* ctx);
/* Launch on an existing cudaStream_t (e.g. torch.cuda.current_stream()). NULL
 * restores the context's own stream. */
int ctraj_set_stream(ctraj_context* ctx, void* cuda_stream);
int ctraj_synchronize(ctraj_context* ctx);

/* Beamline.__post_init__ / sort_elements (beamline.py:17-18,40-45): elements
 * must already be sorted by z0; n_labels counter slots.  Setting the same
 * elements again (bit for bit) changes nothing and costs a comparison. */
int ctraj_set_beamline(ctraj_context* ctx, const ctraj_element* elements,
                       int32_t n_elements, int32_t n_labels);

/* Launch tuning of a context.  No reference counterpart: these are the knobs
 * of this engine's kernels, set by the Python autotuner (ctraj.tuning); the
 * closest reference analogue is its chunking of N_traj into 100 * n_jobs
 * tasks (trajectory_simulator.py:47-49).  Results never depend on them.
 *   chunk_first   RK4 steps of the first lens chunk (molecules still inside the
 *                 lens are compacted between chunks)            default 64
 *   chunk_growth  each chunk is this many percent of the previous  default 200
 *   chunk_max     upper limit of a chunk's steps                  default 1024
 *   front_waves   k_front grid = front_waves x resident CTAs     default 4
 *   lens_mode     FP32 lens pass of runs and sweeps: CTRAJ_LENS_PERSISTENT
 *                 (one launch, lanes refilled, the last molecules compacted
 *                 within each CTA; a sweep's Stark tables share the launch) or
 *                 CTRAJ_LENS_CHUNKED (launches of chunk_* steps, compacted in
 *                 between).  FP64 runs are always chunked.  Results (and ring
 *                 records) do not depend on it.             default persistent
 *   lens_interval persistent mode: RK4 steps between the CTA's compactions
 *                 once the lens queue is empty                   default 256
 *   lens_service  persistent mode: RK4 steps between a warp's finalisations
 *                 and refills of its finished lanes while the queue lasts
 *                 (longer: fewer, fuller finalisation rounds; shorter: less
 *                 idle time of finished lanes)                    default 64
 *   front_threads threads per block of the ballistic front kernel: 128, 256
 *                 or 512                                          default 256
 *   batch_group   ctraj_run_batch: consecutive runs (1-64) whose molecules
 *                 share one persistent lens pass per lens, so the slowest
 *                 molecules of one run (the pass's critical path) overlap the
 *                 bulk of the others.  Applies to FP32 runs without
 *                 per-molecule outputs in persistent lens mode; other runs,
 *                 and batch_group 1, run one at a time.           default 4
 *   lens_threads  molecules per CTA of the persistent FP32 lens pass (one CTA
 *                 per SM) of a run and of a batched sweep: 512, 768 or 1024;
 *                 at one molecule per thread that is 16, 24 or 32 warps per
 *                 SM within a register budget of 128, 80 or 64 per thread
 *                 (sweeps: linear Stark tables staged in shared memory;
 *                 others run 512).                              default 512
 *   lens_molecules molecules each thread of the persistent FP32 lens pass
 *                 steps in turn (1 or 2; with 2 the CTA has lens_threads / 2
 *                 threads, and each RK4 step has a second molecule's
 *                 independent chain to issue against).  default 1
 *                 lens_threads above 512 and lens_molecules 2 apply to runs
 *                 without per-molecule outputs whose table is staged in
 *                 shared memory (lens_molecules 2: hexapole Stark tables);
 *                 others run 512 x 1.
 *   batch_lens_threads lens_threads of the lens passes a batch group shares
 *                 (a group's pass is long enough that more warps per SM pay,
 *                 a single run's is set by its slowest molecule).  default 1024 */
enum { CTRAJ_LENS_PERSISTENT = 0, CTRAJ_LENS_CHUNKED = 1 };

#define CTRAJ_MAX_BATCH_GROUP 64

typedef struct ctraj_tuning {
  int32_t chunk_first;
  int32_t chunk_growth;
  int32_t chunk_max;
  int32_t front_waves;
  int32_t lens_mode;
  int32_t lens_interval;
  int32_t front_threads;
  int32_t batch_group;
  int32_t lens_threads;
  int32_t lens_molecules;
  int32_t batch_lens_threads;
  int32_t lens_service;
} ctraj_tuning;

int ctraj_set_tuning(ctraj_context* ctx, const ctraj_tuning* tuning);
int ctraj_get_tuning(ctraj_context* ctx, ctraj_tuning* tuning);

/* ElectrostaticLens.a_interp / lens_acceleration table (electrostatic_lens.py:174-213),
 * or the cell centres of a Honeycomb (meshes.py:53-62, kind CTRAJ_TABLE_MESH,
 * at least one cell).  Setting the table already set under this id again
 * (knots and coefficients or values bit for bit) changes nothing: the device
 * copies and the lens tables built from it stay. */
int ctraj_set_force_table(ctraj_context* ctx, int32_t table_id,
                          const ctraj_force_table* table);

/* TrajectorySimulator.run_simulation body (trajectory_simulator.py:52-97):
 * propagate, tally into counts, report stats.  Blocks until the counts are on
 * the host. */
int ctraj_run(ctraj_context* ctx, const ctraj_run_args* args,
              ctraj_run_stats* stats);

/*
 * n_runs independent runs, each exactly as ctraj_run(ctx, &args[k], &stats[k])
 * (same counts, stats and outputs), pipelined over two lanes: runs 0, 2, 4, ...
 * on ctx, runs 1, 3, 5, ... on a second context the call keeps inside ctx
 * (same device and beamline, tables and tuning copied from ctx, its own
 * stream, queues and events), each lane driven by its own host thread.  The
 * ballistic front of one lane's run overlaps the other lane's lens pass,
 * whose last molecules leave most SMs idle.  Replaces the caller's loop of one
 * run_simulation per batch of molecules.  Work already queued on ctx's stream
 * is ordered before the batch, and everything the batch does is ordered before
 * later work on ctx's stream.  l2_flush_bytes > 0 writes a context-owned
 * scratch buffer of that many bytes on the lane's stream before each run
 * (benchmarks: no run finds the previous run's data in L2).  stats may be
 * NULL.  Returns the status of the first run (by index) that failed; later
 * runs of the other lane may have completed.
 */
int ctraj_run_batch(ctraj_context* ctx, const ctraj_run_args* args, int32_t n_runs,
                    ctraj_run_stats* stats, uint64_t l2_flush_bytes);

/*
 * Trajectory recording (trajectory_simulator.py:75-76 keeps full Trajectory
 * objects, molecule.py:111-167).  Re-propagates the molecules whose indices
 * are in ids (same ICs as the run that produced them: same seed/offset or the
 * same ics array) and writes every `stride`-th trajectory row plus the last
 * one into rows: (n_ids, max_rows, 10) float64 x, y, z, vx, vy, vz, ax, ay,
 * az, t, on the host.  row_count[k] receives the rows written for ids[k];
 * CTRAJ_EOVERFLOW when a molecule needs more than max_rows.
 */
int ctraj_record(ctraj_context* ctx, const ctraj_run_args* args,
                 const int64_t* ids, int64_t n_ids, int32_t stride,
                 int32_t max_rows, double* rows, int32_t* row_count);

/*
 * z-plane post-processing: post_processing.py find_radial_pos_dist /
 * find_vel_dist (:20-140) for the molecules ids[] of the run described by args
 * (same ICs as that run), evaluated on the device by replaying each molecule.
 * out: (n_ids, 8) float64 x, y, z, vx, vy, vz, status, 0 per molecule, the
 * state at the plane z = z_plane: the trajectory row lying on the plane if
 * there is one (status 2), else the row before the first one past the plane
 * advanced by take_timestep (:9-17, status 1); status 0 (and NaN state) when
 * the molecule's last row is before the plane (the reference skips it).
 */
int ctraj_plane(ctraj_context* ctx, const ctraj_run_args* args, const int64_t* ids,
                int64_t n_ids, double z_plane, double* out);

/*
 * Batched sweep: many lens configurations in one launch sequence.  Replaces
 * the caller's loop of one run_simulation per configuration (the per-state
 * sweep of examples/lens_simulation_different_states.py:136-156 builds one
 * beamline per Stark state and voltage and calls run_simulation on each).
 *
 * The beamline (ctraj_set_beamline) must hold exactly one electrostatic lens
 * with a Stark-spline force law (field_order 1 or 2).  Configuration c differs
 * from it only in the lens: field coefficient alpha[c] (|E| = alpha r^n; the
 * element's p[6]) and Stark table table[c] (a table id set with
 * ctraj_set_force_table, kind CTRAJ_TABLE_STARK_SPLINE).  It propagates
 * n_molecules[c] molecules: molecule j of configuration c is molecule
 * start_c + j of the whole sweep (start_c = sum of the earlier n_molecules),
 * so with device draws it gets Philox counter base->offset + start_c + j,
 * exactly as a ctraj_run of that configuration alone with offset
 * base->offset + start_c.
 *
 * base: precision 32; base->n = the sum of n_molecules; ic_mode as in
 * ctraj_run ((6, base->n) arrays hold the configurations one after another);
 * out_mode CTRAJ_OUT_NONE; base->counts receives the totals over all
 * configurations (n_labels + 1).  counts receives n_configs x (n_labels + 1)
 * int64, row-major.
 *
 * With use_graph != 0 the launch sequence (one ballistic front kernel over all
 * configurations, then per Stark table a fixed sequence of lens chunks on its
 * own stream) is captured once as a CUDA graph and replayed by later calls
 * with the same configurations, initial-condition source and context state.
 * The chunk sequence is sized without a device-to-host read: its last chunk
 * runs every molecule still inside the lens to the end.
 */
/*
 * Ring recording of the molecules lost on one lens.  Replaces keeping full
 * Trajectory objects for apertures of interest (trajectory_simulator.py:75-76,
 * molecule.py:111-167) when the run is too large to replay: during the run
 * itself, every molecule that reaches the lens is staged every `stride` RK4
 * steps; the ones lost on it (label "Inside lens", plus "Lens entrance" for
 * those stopped by the entrance test) are appended to a caller-owned device
 * ring of rows.  A molecule's records are: the lens entrance state (step 0),
 * the state after every stride-th RK4 step, and the state where it was lost.
 * Rows are float32 (x, y, z, vx, vy, vz, t, step); row r of the run is stored
 * at rows[(r mod capacity_rows) * 8].  heads[0] and heads[1] count the rows and
 * molecules appended so far (monotone; the caller zeroes them to start a new
 * ring); molecule m's entry is index[m mod capacity_molecules].  Older
 * records are overwritten once a head passes the capacity.  FP32 runs only;
 * the recorded lens must be the first lens of the beamline.
 */
typedef struct ctraj_ring_entry {
  int64_t molecule;   /* args->offset + index of the molecule in the run (its Philox counter) */
  uint64_t first_row; /* value of heads[0] when its rows were appended          */
  int32_t rows;
  int32_t label;      /* counter slot it was lost on                             */
} ctraj_ring_entry;

typedef struct ctraj_ring {
  float* rows;                /* device: capacity_rows x 8 */
  int64_t capacity_rows;
  ctraj_ring_entry* index;    /* device: capacity_molecules */
  int64_t capacity_molecules;
  unsigned long long* heads;  /* device: 2 counters */
  int32_t stride;             /* RK4 steps between records (>= 1) */
  int32_t lens;               /* element index of the recorded lens */
} ctraj_ring;

/* ctraj_run plus ring recording (args as for ctraj_run, precision 32). */
int ctraj_run_ring(ctraj_context* ctx, const ctraj_run_args* args,
                   const ctraj_ring* ring, ctraj_run_stats* stats);

#define CTRAJ_MAX_SWEEP_CONFIGS 65536
typedef struct ctraj_sweep {
  int32_t n_configs;
  int32_t use_graph;
  const int64_t* n_molecules;  /* n_configs */
  const double* alpha;         /* n_configs: lens field coefficient */
  const int32_t* table;        /* n_configs: Stark table id */
} ctraj_sweep;

int ctraj_run_sweep(ctraj_context* ctx, const ctraj_sweep* sweep,
                    const ctraj_run_args* base, int64_t* counts,
                    ctraj_run_stats* stats);

/*
 * Soft transmission and its gradient.  No reference counterpart: the
 * reference has only hard counts (Counter, trajectory_simulator.py:106-158);
 * this makes the beamline differentiable so it can be tuned by gradient
 * descent.  Every hard aperture test (the circular apertures in front of the
 * lens and behind it, at both of their planes, the lens entrance, the bore
 * test after each RK4 step) becomes the weight sigmoid((R - r) / width); the
 * loss is the mean over molecules of the product of their weights.  Molecules
 * whose log weight falls below log_floor are dropped (counted as weight 0).
 * Behind the lens a molecule flies with gravity alone from its state after
 * the last RK4 step (z0 + N dz) to each aperture plane: the reference's exit
 * snap to z1 with the last step's lens force (electrostatic_lens.py:74-77,
 * at most dz / 2) is taken as part of that flight.
 *
 * Beamline: circular apertures, then exactly one electrostatic lens with a
 * Stark spline table and field order 2 (|E| = 3 V r^2 / R^3, R = p[4]), then
 * circular apertures (any diameter; an infinite one is a plane without test).
 *
 * params[CTRAJ_SOFT_NPARAMS]: lens voltage, lens z0 (the lens moves, its
 * length stays), the radius of the circular aperture at element index
 * args->aperture (in front of the lens or behind it; ignored when -1), the clip radius of the lens bore (the field
 * radius R stays fixed), and the standard deviations of vx and vy (replacing
 * those of args->vdist).  Initial conditions: Philox draws exactly as ctraj_run
 * (CTRAJ_IC_DEVICE_DRAW), or the caller's unit normals (CTRAJ_IC_HOST:
 * normals = (5, n) float64 n_vx, n_vy, n_vz, n_x, n_y; v = mu + sigma n,
 * x = sigma_x n_x, y = sigma_y n_y).
 *
 * With want_grad the gradient d loss / d params is the exact derivative of
 * the computation (discrete adjoint): lens states are checkpointed every
 * `checkpoint` RK4 steps (1..64) and each segment is recomputed in the
 * backward pass.  Blocks until the result is on the host.
 */
#define CTRAJ_SOFT_NPARAMS 6
enum {
  CTRAJ_SOFT_V = 0,
  CTRAJ_SOFT_LENS_Z0 = 1,
  CTRAJ_SOFT_APERTURE_R = 2,
  CTRAJ_SOFT_BORE_R = 3,
  CTRAJ_SOFT_SIGMA_VX = 4,
  CTRAJ_SOFT_SIGMA_VY = 5
};

typedef struct ctraj_soft_args {
  int64_t n;
  int32_t precision;          /* 32 or 64 */
  int32_t ic_mode;            /* CTRAJ_IC_DEVICE_DRAW or CTRAJ_IC_HOST (unit normals) */
  const double* normals;      /* CTRAJ_IC_HOST: (5, n), host memory */
  uint64_t seed;
  uint64_t offset;
  ctraj_distribution xdist;   /* CTRAJ_DIST_GAUSSIAN_POSITION */
  ctraj_distribution vdist;   /* CTRAJ_DIST_GAUSSIAN_VELOCITY */
  double g;
  double width;               /* sigmoid width (m) */
  double log_floor;           /* e.g. -30 */
  int32_t aperture;           /* element index of the aperture parameter, or -1 */
  int32_t checkpoint;         /* RK4 steps between lens checkpoints, 1..64 */
  int32_t want_grad;
  int32_t timing;
} ctraj_soft_args;

typedef struct ctraj_soft_result {
  double loss;
  double grad[CTRAJ_SOFT_NPARAMS];
  int64_t lens_molecules;     /* molecules that reached the lens above log_floor */
  int64_t lens_steps;         /* RK4 steps of the forward pass */
  int64_t dropped;            /* molecules dropped below log_floor */
  int64_t bad_steps;          /* molecules with an unusable rint(L/dz) (dropped) */
  int32_t kernels;
  int32_t timed;
  float front_ms;             /* ballistic part */
  float lens_ms;              /* lens forward (and backward) */
} ctraj_soft_result;

int ctraj_soft_transmission(ctraj_context* ctx, const ctraj_soft_args* args,
                            const double* params, ctraj_soft_result* result);

/*
 * Allocation-free run.  This entry point has no counterpart in the reference.
 *
 * ctraj_run_noalloc propagates molecules exactly as ctraj_run does with its
 * default tuning (same kernels: the ballistic front, the lens-entrant
 * ordering and the persistent lens pass with compaction interval 256; same
 * counts, stats and per-molecule outputs, bit for bit) but needs no context
 * and allocates no device memory: its scratch (lens queues, queue counters,
 * tallies, the FP32 lens tables, the lens-entrant order) lives in one
 * file-scope __device__ array of CTRAJ_NOALLOC_SCRATCH_BYTES that every GPU
 * which loads libctraj.so holds until the process exits.  It is for callers
 * that cannot allocate device memory while they run: an application that
 * hands this library a fixed device-memory budget at start-up and owns every
 * allocation itself, or a service that must not call cudaMalloc/cudaFree on
 * its request path because those calls synchronize the whole device and
 * stall the other work on it.
 *
 * Limits: precision 32 only; at most CTRAJ_NOALLOC_MAX_MOLECULES molecules per
 * call and at most CTRAJ_NOALLOC_MAX_INTERVALS FP32 table entries over all
 * lenses and meshes (larger inputs are rejected with CTRAJ_EINVAL before any
 * CUDA call); initial conditions drawn on the device or given in device
 * memory (CTRAJ_IC_DEVICE); per-molecule outputs, if any, in device memory
 * (CTRAJ_OUT_DEVICE); counts are written to the host array args->counts.
 * Runs on the calling thread's current device and context and on
 * `cuda_stream` (NULL = the legacy default stream), and returns after the
 * counts are on the host.
 *
 * The array's device address is looked up (cudaGetSymbolAddress) by the first
 * call in each CUDA context, with that context current: the first call on a
 * device, the first call in a context created with cuCtxCreate, and the first
 * call after cudaDeviceReset (which replaces the primary context).  Make that
 * first call before any stream capture.  All calls share the one array and
 * each overwrites it (it starts every call by clearing its counters), so calls
 * that overlap on the GPU (from two host threads, or on two streams) race:
 * serialize them.
 */
#define CTRAJ_NOALLOC_MAX_MOLECULES 131072
#define CTRAJ_NOALLOC_MAX_INTERVALS 16384 /* FP32 table entries over all lenses (one per knot interval, two in the linear Stark form) + honeycomb cells */
#define CTRAJ_NOALLOC_SCRATCH_BYTES (32u << 20)
int ctraj_run_noalloc(const ctraj_element* elements, int32_t n_elements,
                      int32_t n_labels, const ctraj_force_table* tables,
                      int32_t n_tables, const ctraj_run_args* args,
                      void* cuda_stream, ctraj_run_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* CTRAJ_H_ */
