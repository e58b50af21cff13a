/*
 * ts_fvm.h -- C ABI of the GB300-native explicit finite-volume step.
 *
 * This is the drop-in boundary for TurboStructred's hot path: the explicit
 * FVM residual and stage update of ExplicitRungeKuttaFVM<R>
 * (src/Methods/ExplicitRungeKuttaFVM.h:15-1493) together with the Kernel
 * state, ghost fill, CFL time step and update it drives (src/kernel/kernel.h).
 * Plain C types only: no CUDA, C++ or torch types cross this boundary.
 *
 * Plugin selection keeps the reference's enum values
 * (src/Methods/MethodConfiguration.h:5-23,
 *  src/BoundaryConditions/BoundaryConditionConfiguration.h:12-19); values this
 * project adds (HLLC, stiffened gas, precision modes) are appended after them.
 *
 * Errors: every call returns a ts_status; ts_last_error() gives the message
 * of the most recent failure on the calling thread.  Handles are not
 * thread-safe: one host thread drives one handle.  Each handle owns one CUDA
 * stream on its device.
 */
#ifndef TS_FVM_H
#define TS_FVM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TS_FVM_ABI_VERSION 5

typedef enum ts_status {
    TS_OK = 0,
    TS_ERR_INVALID = 1,      /* bad argument or configuration */
    TS_ERR_UNSUPPORTED = 2,  /* valid in the reference but not built here */
    TS_ERR_CUDA = 3,         /* CUDA runtime error (message has details) */
    TS_ERR_NO_MEMORY = 4,    /* device or host allocation failed / budget */
    TS_ERR_NUMERIC = 5,      /* NaN, rho <= 0 or p <= 0 detected */
    TS_ERR_TIMEOUT = 6,      /* a bounded device wait gave up */
    TS_ERR_BUSY = 7,         /* resource in use (e.g. server full) */
    TS_ERR_NOT_FOUND = 8     /* unknown request id */
} ts_status;

/* Reconstruction (MethodConfiguration.h:5-10) */
enum {
    TS_RECON_PIECEWISE_CONSTANT = 0,
    TS_RECON_LINEAR_2POINTS = 1,
    TS_RECON_ENO2_2POINTS = 2,
    TS_RECON_LINEAR_2POINTS_LIMITED = 3
};
/* RPSolver (MethodConfiguration.h:13-17) + HLLC (new).  Godunov (the exact
   solver) runs on the FP64 path with the ideal-gas EOS. */
enum { TS_RS_GODUNOV = 0, TS_RS_ROE_PIKE = 1, TS_RS_NONE = 2, TS_RS_HLLC = 3 };
/* LimiterType (MethodConfiguration.h:20-23) */
enum { TS_LIM_BARTH_JESPERSEN = 0, TS_LIM_VENKATAKRISHNAN = 1 };
/* BoundaryConditionType (BoundaryConditionConfiguration.h:12-19) */
enum {
    TS_BC_WALL = 0,
    TS_BC_SYMMETRY = 1,
    TS_BC_MOVING_WALL = 2,
    TS_BC_SUBSONIC_INLET = 3,
    TS_BC_SUBSONIC_OUTLET = 4,
    TS_BC_NATURAL = 5
};
/* Equation of state: ideal gas (the reference's, RoeSolverPerfectGasEOS.h:23)
   and stiffened gas p = (gamma-1) rho e - gamma p_inf (new). */
enum { TS_EOS_IDEAL_GAS = 0, TS_EOS_STIFFENED_GAS = 1 };
/* Precision: all-FP64 (bit-for-bit with the reference), or FP32
   reconstruction/EOS/flux with FP64 state, stage accumulation and dt. */
enum { TS_PRECISION_FP64 = 0, TS_PRECISION_MIXED = 1 };
/* Host state layouts for ts_set_state / ts_get_state. */
enum {
    TS_LAYOUT_INTERIOR = 0,   /* interior cells only, x fastest, 5 doubles per cell */
    TS_LAYOUT_WITH_GHOSTS = 1 /* the reference's Kernel::values array (kernel.h:88-96) */
};
/* Health flags reported in ts_step_info.health */
enum {
    TS_HEALTH_NAN = 1u,
    TS_HEALTH_NEG_DENSITY = 2u,
    TS_HEALTH_NEG_PRESSURE = 4u,
    TS_HEALTH_RIEMANN = 8u, /* the exact (Godunov) solver's p* iteration did not converge at some face */
    TS_HEALTH_TIMEOUT = 16u /* a bounded wait inside a kernel gave up (the step's results are not valid) */
};

/* BlockNode (KernelConfiguration.h:10-19): stretched-grid block start. */
typedef struct ts_block_node {
    double pos;
    double q_com;
    int32_t n_cells;
    int32_t reserved;
} ts_block_node;

/* BoundaryConditionConfiguration (BoundaryConditionConfiguration.h:21-35). */
typedef struct ts_bc_config {
    int32_t type;
    int32_t reserved;
    double density;
    double velocity[3];
    double pstatic;
    double temperature;
} ts_bc_config;

/* Extra boundary-condition configurations a position-dependent side can
   select (ts_config.bc_kinds). */
#define TS_MAX_BC_KINDS 8

/* KernelConfiguration (KernelConfiguration.h:21-93) with its
   MethodConfiguration (MethodConfiguration.h:26-37), reduced to the fields the
   explicit inviscid step reads.  One BC per domain side, in the order
   x-, x+, y-, y+, z-, z+ (the reference's trivial-marker DomainBCinfo),
   unless the side has a marker array (see bc_marker below). */
typedef struct ts_config {
    int32_t abi_version;   /* TS_FVM_ABI_VERSION */
    int32_t n_dims;        /* nDims */
    int32_t nx, ny, nz;    /* nX, nY, nZ */
    int32_t periodic[3];   /* isPeriodicX/Y/Z */
    double length[3];      /* LX, LY, LZ */
    int32_t n_blocks[3];   /* CompressionX/Y/Z sizes; 0 = uniform */
    int32_t reserved0;
    const ts_block_node* blocks[3];
    double gamma;          /* Gamma */
    int32_t eos;           /* TS_EOS_* */
    int32_t reserved1;
    double p_inf;          /* stiffened-gas constant (0 for ideal gas) */
    int32_t reconstruction;  /* ReconstructionType */
    int32_t riemann_solver;  /* RiemannProblemSolver */
    int32_t limiter;         /* GeneralLimitter */
    int32_t rk_order;        /* RungeKuttaOrder (the reference always runs 1 stage) */
    double cfl;              /* CFL */
    double eps;              /* Eps (Harten entropy fix) */
    int32_t max_iteration;   /* MaxIteration */
    int32_t reserved2;
    double max_time;         /* MaxTime */
    double save_solution_time; /* SaveSolutionTime: clips dt (ExplicitRungeKuttaFVM.h:1433) */
    double save_slice_time;    /* SaveSliceTime: clips dt (ExplicitRungeKuttaFVM.h:1434) */
    ts_bc_config bc[6];
    int32_t precision;       /* TS_PRECISION_* */
    int32_t device;          /* CUDA device ordinal */
    /* Source terms (Kernel::ProcessExternalForces / ProcessExternalAcceleration,
       kernel.h:941-989), added to the residual after the face fluxes. */
    int32_t external_force;        /* IsExternalForceRequared: R_mom += V Sigma, R_E += V Sigma.u */
    int32_t uniform_acceleration;  /* IsUnifromAccelerationRequared: R_mom += rho V g, R_E += V rho g.u */
    double sigma[3];               /* Sigma */
    double acceleration[3];        /* UniformAcceleration */
    /* Viscous flow (ExplicitRungeKuttaFVM.h:81-874, :1161-1170): with
       `viscous` set, velocity gradients (central in the interior, least
       squares at non-periodic boundaries) give the stress-tensor face fluxes
       subtracted from the convective ones.  `viscosity` (gas viscosity mu)
       also enters the spectral radius of every step, viscous or not
       (:1239-1248).  FP64 precision only (TS_ERR_UNSUPPORTED otherwise). */
    int32_t viscous;               /* IsViscousFlow */
    /* Mixed precision only: also form the volume-weighted L1 residual norms
       of every step (kernel.h:326) as FP64 sums of V |R| over the FP32
       residual.  The FP64 path always forms them. */
    int32_t residual_norms;
    double viscosity;              /* Viscosity */
    /* Position-dependent boundary conditions: a domain side carrying several
       BCs (DomainBCinfo::isComplex and getMarker,
       BoundaryConditionConfiguration.h:43-66, honoured by
       Kernel::InitBoundaryConditions, kernel.h:284-316).  bc_kinds[0 ..
       n_bc_kinds) are further BC configurations (the reference's
       MyConditions entries).  A side whose bc_marker[side] is non-NULL takes,
       at each of its boundary faces, bc_kinds[bc_marker[side][f]] in place of
       bc[side]; the caller evaluates its marker function at the faces'
       centres (as ComputeResidual does, ExplicitRungeKuttaFVM.h:1193-1209)
       and the same marker serves the ghost cells of that face's row.  Faces
       f are numbered by the side's two tangential cell indices, the lower
       axis fastest: x sides j + ny*k, y sides i + nx*k, z sides i + nx*j
       (ny*nz, nx*nz, nx*ny entries; inactive axes have one cell).  The arrays
       are copied by ts_create.  Single problems only (batches, served solves
       and ts_advance_noalloc refuse them with TS_ERR_UNSUPPORTED). */
    int32_t n_bc_kinds;
    int32_t reserved4;
    ts_bc_config bc_kinds[TS_MAX_BC_KINDS];
    const uint8_t* bc_marker[6];
} ts_config;

/* StepInfo (kernel.h:31-39) plus a health word. */
typedef struct ts_step_info {
    int32_t iteration;
    uint32_t health;
    double time;
    double dt;
    double next_solution_time;
    double next_slice_time;
    double residual[5];  /* volume-weighted L1 residual norms sum V |R| of the last step
                            (kernel.h:326); the FP64 path forms them every step, the
                            mixed path when ts_config.residual_norms is set (else zeros) */
} ts_step_info;

typedef struct ts_handle ts_handle;

/* Replaces `new ExplicitRungeKuttaFVM<R>` + Kernel::Init (kernel.h:178-281)
   and the factory CreateKernel (ExplicitRungeKuttaFVM.h:1496-1513): grid,
   boundary conditions and method set-up, device state allocation. */
ts_status ts_create(const ts_config* cfg, ts_handle** out);

/* Releases device memory and the stream (Kernel::Finalize, kernel.h:1879). */
void ts_destroy(ts_handle* h);

/* Writes the conserved state, like Kernel::SetInitialConditions
   (kernel.h:125-146) for a point-sampled field, from a host array. */
ts_status ts_set_state(ts_handle* h, const double* values, int32_t layout);

/* Same from a device pointer on the handle's device (no host copy).  The
   handle reads it on its own stream, which does not wait for the caller's
   streams: work that writes device_values must have completed before the
   call (synchronize its stream).  The call returns after the read, so the
   buffer may be reused at once. */
ts_status ts_set_state_device(ts_handle* h, const double* device_values, int32_t layout);

/* Reads Kernel::values back (kernel.h:88). */
ts_status ts_get_state(ts_handle* h, double* values, int32_t layout);

/* Same into a device buffer on the handle's device (no host copy and no
   staging buffer; the state of a grid too large for host memory can be
   read this way).  Returns after the buffer is written; work of the caller
   that uses device_values may run on any stream after the call. */
ts_status ts_get_state_device(ts_handle* h, double* device_values, int32_t layout);

/* n_steps calls of ExplicitRungeKuttaFVM::IterationStep (:1440-1491). */
ts_status ts_step(ts_handle* h, int32_t n_steps, ts_step_info* info);

/* Device timing of n steps, for benchmarks: CUDA events recorded on the
   handle's stream around the whole run and around every kernel launch of up
   to 64 evenly spaced steps (launched one by one, not from a graph).
   Per-kernel times are averages per launch over those steps; names identify
   the kernels of one step in launch order. */
#define TS_MAX_KERNELS 16
typedef struct ts_timing {
    double total_ms;
    int32_t n_kernels;        /* kernels per step */
    int32_t launches;         /* kernel launches in the timed region */
    double kernel_ms[TS_MAX_KERNELS];
    char kernel_name[TS_MAX_KERNELS][32];
} ts_timing;
ts_status ts_step_timed(ts_handle* h, int32_t n_steps, ts_step_info* info, ts_timing* timing);

/* Kernel::Run (kernel.h:1635-1876): steps until MaxIteration or MaxTime,
   with the reference's termination order and dt overshoot. */
ts_status ts_run(ts_handle* h, ts_step_info* info);

/* Current StepInfo; and setting it (resume from a checkpoint,
   Kernel::LoadSolution kernel.h:1031-1079 restores Time). */
ts_status ts_get_step_info(ts_handle* h, ts_step_info* info);
ts_status ts_set_step_info(ts_handle* h, const ts_step_info* info);

/* Launch shape of the mixed-precision fused kernel: the tile (threads per
   CTA along x and y; compiled shapes: 3D 32x8, 16x16, 32x16, each thread one
   cell, marching z; 2D 260, 132, 68 one-row tiles marching y; 1D 512, 256,
   128; one-row tiles own tx - 4 cells) and the number of chunks each tile
   column's march is cut into (0 = chosen from the grid and the SM count).
   Every face flux is a function of its two cells only; other tiles are
   other compiled instances and agree to FP32 rounding.
   TS_ERR_UNSUPPORTED for the FP64 path or an uncompiled tile. */
ts_status ts_set_tile(ts_handle* h, int32_t tx, int32_t ty, int32_t z_chunks);

/* Waits for all work queued on the handle's stream. */
ts_status ts_synchronize(ts_handle* h);

/* Cell centres and sizes with one ghost layer per active axis, exactly as
   Grid::InitLocal accumulates them (grid.h:124-344).  Host-only; any pointer
   may be NULL.  Array lengths are nx+2, (ny+2 | 1), (nz+2 | 1). */
ts_status ts_grid_coordinates(const ts_config* cfg, double* x, double* hx, double* y, double* hy,
                              double* z, double* hz);

/* Number of doubles in a host state array of the given layout. */
size_t ts_state_doubles(const ts_config* cfg, int32_t layout);

/* Synthetic initial states of the benchmark scenarios (host-only, no GPU),
   point-sampled at the grid's cell centres with a counter-based hash RNG of
   (seed, i, j, k), written in TS_LAYOUT_INTERIOR order.  See ts_scenario. */
enum {
    TS_SCENARIO_SHOCK_TUBE = 0, /* params: x0, rhoL, uL, pL, rhoR, uR, pR */
    TS_SCENARIO_SHEAR_LAYER = 1, /* params: rho_in, rho_out, u, p, noise amplitude */
    TS_SCENARIO_BLAST = 2,       /* params: rho, p_out, p_in, radius, noise amplitude */
    TS_SCENARIO_QUADRANTS = 3    /* params: 4 x (rho, u, v, p) for quadrants ++,-+,--,+- */
};
ts_status ts_fill_scenario(const ts_config* cfg, int32_t scenario, uint64_t seed, const double* params,
                           int32_t n_params, double* values);

/* The hash RNG the scenarios use: uniform double in [0,1). */
double ts_hash_uniform(uint64_t seed, int64_t i, int64_t j, int64_t k);

/* ---------------------------------------------------------------------------
   Solution files in the reference's formats, for one domain (the reference's
   rank 0).
   --------------------------------------------------------------------------- */

/* Kernel::SaveSolution (kernel.h:992-1028): binary file of the current time
   (double), the rank (int32, 0) and the interior cells' conserved values
   (k, j, i order, x fastest, 5 doubles each). */
ts_status ts_save_solution(ts_handle* h, const char* path);

/* Kernel::LoadSolution (kernel.h:1029-1079): reads such a file into the state
   and sets the time; the iteration count is kept and the next snapshot times
   restart after the loaded time, as the reference does.  Files whose first
   block is not rank 0 are refused (TS_ERR_UNSUPPORTED). */
ts_status ts_load_solution(ts_handle* h, const char* path);

/* Kernel::SaveSolutionToTecplot (kernel.h:1082-1413): Tecplot text, byte-
   identical to the reference's for the same state.  molar_mass and
   gas_constant are KernelConfiguration::MolarMass and ::UniversalGasConstant
   (defaults 0 and 8.3144598; they only enter the temperature column).
   async != 0 snapshots the state and writes the file on a worker thread;
   ts_wait_writes joins the pending writes (ts_destroy does too). */
ts_status ts_save_tecplot(ts_handle* h, const char* path, double molar_mass, double gas_constant, int32_t async);
ts_status ts_wait_writes(ts_handle* h);

/* The same three formats from and to host arrays (TS_LAYOUT_INTERIOR), with
   no device work. */
ts_status ts_write_solution_file(const ts_config* cfg, const double* values, double time, const char* path);
ts_status ts_read_solution_file(const ts_config* cfg, const char* path, double* values, double* time);
ts_status ts_write_tecplot_file(const ts_config* cfg, const double* values, double time, double molar_mass,
                                double gas_constant, const char* path);

/* ---------------------------------------------------------------------------
   Batches: many independent problems of different sizes advanced together.
   No counterpart in the reference (one Kernel per process there); each
   problem follows Kernel::Run semantics with its own dt (CFL minimum over its
   own cells) and its own MaxTime / MaxIteration.  All problems of a batch are
   1D or 2D, mixed precision; solvers and equations of state may differ.
   One stage of every unfinished problem is one launch of the fused kernel per
   (dimension, Riemann solver) present, over a work list of (problem, tile)
   items, largest problems first; stage
   chunks are replayed from CUDA graphs while the membership is unchanged.
   --------------------------------------------------------------------------- */
typedef struct ts_batch ts_batch;

/* memory_budget: bytes of device memory for all problem states (one arena). */
ts_status ts_batch_create(int32_t device, size_t memory_budget, ts_batch** out);
void ts_batch_destroy(ts_batch* b);

/* Adds a problem with its initial state (host, TS_LAYOUT_INTERIOR); cfg must
   be 1D/2D with TS_PRECISION_MIXED.  TS_ERR_NO_MEMORY when the arena cannot
   hold it (nothing is changed then).  *id identifies it until removed. */
ts_status ts_batch_add(ts_batch* b, const ts_config* cfg, const double* values, int32_t* id);

/* Device bytes a problem would take in a batch arena (0: not batchable). */
size_t ts_batch_problem_bytes(const ts_config* cfg);

/* n_stages stages of every unfinished problem (finished ones are skipped). */
ts_status ts_batch_step(ts_batch* b, int32_t n_stages);

/* The same split in two: ts_batch_launch queues the stages and returns;
   ts_batch_wait waits for them and refreshes every problem's step info
   (*active: problems still running).  Between the two, ts_batch_add uploads
   and ts_batch_get / ts_batch_remove of finished problems run beside the
   queued stages (their own streams). */
ts_status ts_batch_launch(ts_batch* b, int32_t n_stages);
ts_status ts_batch_wait(ts_batch* b, int32_t* active);

/* Stages until every problem has finished (MaxTime or MaxIteration), at most
   max_stages (<= 0: no limit).  *active receives the problems still running.
   A problem whose state turns non-physical (NaN, density <= 0) is stopped
   and reported finished; ts_batch_get returns its health flags. */
ts_status ts_batch_run(ts_batch* b, int32_t max_stages, int32_t* active);

/* Ids of finished problems not yet collected (up to cap); *n receives the count. */
ts_status ts_batch_finished(ts_batch* b, int32_t* ids, int32_t cap, int32_t* n);

/* State (TS_LAYOUT_INTERIOR, may be NULL) and step info of a problem. */
ts_status ts_batch_get(ts_batch* b, int32_t id, double* values, ts_step_info* info);

/* Frees a problem's slot and memory. */
ts_status ts_batch_remove(ts_batch* b, int32_t id);

/* Launch shape for the problems of dimension nd: tx = threads of the
   one-row tile along x (1D: 512, 256, 128; 2D: 260, 132, 68; the tile owns
   tx - 4 cells), or 0 to pick per problem from its x extent; ty is ignored;
   and CTAs per SM of the persistent grid (0 = as many as fit). */
ts_status ts_batch_set_tile(ts_batch* b, int32_t nd, int32_t tx, int32_t ty, int32_t ctas_per_sm);

/* The batch's tail mode (on by default): once every unfinished problem is
   1D, fits one thread-block cluster (at most 16 x 508 cells) and all of them
   together fit the GPU at once, each launch advances every problem by up to
   the requested number of stages in the cluster tail kernel, with the state
   kept on chip between stages; results are identical to the stage-by-stage
   path.  enable = 0 keeps the stage-by-stage path throughout. */
ts_status ts_batch_set_tail(ts_batch* b, int32_t enable);

/* Autotuner: times `stages` stages of the current batch for the per-problem
   policy and every compiled tile, each at several CTA counts, restoring the
   problems' states after each trial, and keeps the fastest; *tx (0: per
   problem), *ty, *ctas_per_sm receive the choice for the batch's dominant
   dimension. */
ts_status ts_batch_autotune(ts_batch* b, int32_t stages, int32_t* tx, int32_t* ty, int32_t* ctas_per_sm);

/* Totals since creation: cell-updates done, stages launched, kernel launches. */
ts_status ts_batch_stats(ts_batch* b, double* cell_updates, int64_t* stages, int64_t* launches);

/* ---------------------------------------------------------------------------
   Served solves: a request loop over one batch.  No counterpart in the
   reference.  Requests (1D/2D, mixed precision, any EOS / solver /
   reconstruction) are submitted from any thread and queue in arrival order;
   a worker thread admits queued solves (in arrival order, or least work
   first) whenever the batch arena has room and the caps on admitted cells
   and solves allow, advances all admitted solves together in chunks of
   stages, and retires each one as it reaches its MaxTime / MaxIteration.  Requests that arrive while others run
   join at the next chunk boundary (continuous batching): each result is that
   of the problem alone in a batch, bit for bit.
   --------------------------------------------------------------------------- */
typedef struct ts_server ts_server;

typedef struct ts_request_times {
    double submit_s;   /* seconds since the server was created */
    double admit_s;    /* state uploaded, first chunk pending */
    double finish_s;   /* retired: final state read back */
} ts_request_times;

typedef struct ts_server_stats {
    int64_t submitted, admitted, completed, rejected;
    int64_t queued, active;            /* right now */
    int64_t stages, launches;          /* batch totals */
    double cell_updates;               /* of all solves, retired or running */
    double busy_s;                     /* worker time advancing admitted solves */
    double admit_s, retire_s;          /* worker time uploading admitted / reading back finished solves */
    double latency_p50_ms, latency_p99_ms, latency_max_ms;  /* submit -> finish, completed solves */
    double wait_p50_ms, wait_p99_ms;   /* submit -> admit */
    size_t bytes_budget, bytes_in_use;
    ts_status worker_status;           /* first error the worker met (TS_OK if none) */
} ts_server_stats;

/* Admission order of queued solves. */
enum {
    TS_SERVE_FIFO = 0,            /* arrival order; the head waits for room */
    TS_SERVE_SHORTEST_FIRST = 1   /* least work first (cells x MaxIteration, or cells when
                                     only MaxTime bounds it), arrival order among equals */
};

typedef struct ts_server_config {
    int32_t device;
    int32_t order;          /* TS_SERVE_* */
    size_t memory_budget;   /* bytes of device memory for admitted solves */
    int64_t max_cells;      /* cells admitted at once (0: memory is the only limit).  The
                               GPU's throughput saturates at a few million cells in
                               flight; admitting more only slows every solve down */
    int32_t max_active;     /* admitted solves at once (0: no cap) */
    int32_t reserved;
    double chunk_ms;        /* target duration of one chunk of stages (0: 2 ms) */
} ts_server_config;

ts_status ts_server_create(const ts_server_config* cfg, ts_server** out);
/* Stops the worker (solves in flight are dropped) and frees everything. */
void ts_server_destroy(ts_server* s);

/* Queues a solve; cfg and values are copied.  keep_state = 0 keeps only the
   step info and times (no final state).  TS_ERR_UNSUPPORTED for a problem a
   batch cannot hold, TS_ERR_NO_MEMORY for one larger than the whole budget. */
ts_status ts_server_submit(ts_server* s, const ts_config* cfg, const double* values, int32_t keep_state,
                           int32_t* request_id);

/* Waits up to timeout_ms (< 0: forever) for a request; TS_ERR_TIMEOUT if it
   has not finished.  On success copies the final state (if kept and values is
   not NULL), its step info and times, and forgets the request. */
ts_status ts_server_wait(ts_server* s, int32_t request_id, int32_t timeout_ms, double* values, ts_step_info* info,
                         ts_request_times* times);

/* Waits up to timeout_ms (< 0: forever) until nothing is queued or running. */
ts_status ts_server_drain(ts_server* s, int32_t timeout_ms);

ts_status ts_server_stats_get(ts_server* s, ts_server_stats* out);

/* Advance a state by n_steps of the mixed-precision fused step without
   allocating any device memory.  No counterpart in the reference: this is
   for callers that are not allowed to call cudaMalloc themselves or through
   us -- code embedded in a host application that owns every byte of device
   memory through its own pool or budget, or a latency-critical loop where an
   allocation's implicit synchronisation and unpredictable cost are not
   acceptable.
     cfg       problem set-up; precision must be TS_PRECISION_MIXED.
     state_in  device pointer, TS_LAYOUT_INTERIOR doubles (caller-owned).
     state_out device pointer, same layout (may equal state_in).
     stream    a cudaStream_t, or NULL for the legacy default stream.  Every
               upload, clear and kernel of the call is queued on it, so the
               call is ordered after work already queued there.
     info      optional; its time, iteration and snapshot times are the
               starting point and it receives the step info at the end.  A
               fresh run (info NULL, or iteration 0 at time 0, e.g. a
               zero-filled struct) starts the snapshot schedule at
               cfg->save_solution_time / save_slice_time as ts_create does;
               otherwise next_solution_time / next_slice_time are taken
               from info, so a continued run passes back what it received.
               residual[] receives the norms when cfg->residual_norms is set
               (formed in FP64 from the FP32 residual), else zeros.
   Every call works in one file-scope scratch array of TS_NOALLOC_MAX_PLANE
   elements per variable plane (about 38 MB, resident on every GPU that has
   loaded this library, until the process exits): grids whose padded planes
   exceed it are rejected with TS_ERR_INVALID.  The first call on a device
   looks up that array's device address, so make it before any stream
   capture.  Each call waits on the host for its own work on `stream` to
   finish before it returns (it reads the step count and time back).  All
   calls share the array and leave their data in it; calls that overlap on
   the GPU (other streams, other host threads) race on it. */
#define TS_NOALLOC_MAX_PLANE 262144
ts_status ts_advance_noalloc(const ts_config* cfg, const double* state_in, double* state_out, int32_t n_steps,
                             void* stream, ts_step_info* info);

const char* ts_last_error(void);
const char* ts_status_string(ts_status s);

#ifdef __cplusplus
}
#endif
#endif
