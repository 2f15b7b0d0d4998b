/* dcgpu: GB300-native implicit-step engine for DuneCopasi diffusion-reaction models.
 *
 * C ABI of the drop-in boundary.  Every entry point returns an int status (DC_OK = 0);
 * no C++ exception crosses this boundary.  dc_last_error() gives the message of the
 * last failure on the calling thread.  One host thread per model handle.
 *
 * Each entry point names the reference interface it replaces (paths inside the
 * dune-copasi source tree).
 */
#ifndef DCGPU_H
#define DCGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  DC_OK = 0,
  DC_ERR_DIVERGED = 1, /* Newton or linear solve did not converge (PDELab::ErrorCondition) */
  DC_ERR_DT_MIN = 2,   /* time step reached time_step_min (stepper.hh:371-382) */
  DC_ERR_TIMEOUT = 3,  /* iteration cap reached */
  DC_ERR_CONFIG = 4,   /* configuration error (format_exception(IOError...)) */
  DC_ERR_CUDA = 5,
  DC_ERR_ARGUMENT = 6,
  DC_ERR_INTERNAL = 7
};

typedef struct dc_model dc_model;

typedef struct dc_model_info {
  int32_t dim;          /* grid dimension */
  int32_t n_species;    /* scalar fields over all compartments */
  int32_t n_compartments;
  int32_t block_size;   /* species per block row on the device */
  int64_t n_vertices;
  int64_t n_elements;
  int64_t n_dof;        /* reference DOF count */
  int64_t n_block_rows;
  int64_t n_blocks;     /* stored BSR blocks */
} dc_model_info;

typedef struct dc_step_info {
  double time;          /* time after the step */
  double dt_used;       /* step size that succeeded */
  int32_t newton_iterations;  /* Newton iterations in this step, all stages */
  int32_t linear_iterations;  /* Krylov iterations in this step */
  int32_t failed_attempts;    /* attempts rejected before success */
  int32_t status;
  double device_ms;           /* CUDA-event time of the step on the model's stream */
} dc_step_info;

typedef void (*dc_callback)(const dc_model* model, double time, void* user);

/* Replaces DiffusionReaction::make_model + Model::make_state + make_step_operator
 * (dune/copasi/model/diffusion_reaction/factory.hh:46-136, model/model.hh:24-101,
 * model_single_compartment.impl.hh:195-232).  `ini_text` is the configuration file
 * content; `overrides` holds "key=value" lines (the CLI's --key=value, src/dune_copasi.cc:
 * 270-288) or is NULL.  The state is initialised from the initial conditions. */
int dc_model_create(const char* ini_text, const char* overrides, dc_model** out);
/* Value of a configuration key after the overrides (Dune::ParameterTree::get on the model's
 * configuration): copies the value into buf (NUL-terminated, truncated to len); returns
 * DC_ERR_CONFIG when the key is absent.  For callers such as the CLI's writer / reduce
 * settings (src/dune_copasi.cc:403-423). */
int dc_config_get(const dc_model* model, const char* key, char* buf, size_t len);
int dc_model_destroy(dc_model* model);
int dc_model_info_get(const dc_model* model, dc_model_info* info);

/* species metadata (names in configuration order, compartment-major) */
int dc_species_name(const dc_model* model, int32_t species, char* buf, size_t len);
int dc_species_size(const dc_model* model, int32_t species, int64_t* n_vertices);
int dc_species_vertices(const dc_model* model, int32_t species, int64_t* vertex_ids, size_t n);
/* vertex coordinates, n_vertices x dim row-major (the grid's Geometry::corner values the
 * reference's nodal interpolation evaluates at, model/interpolate.hh:21-78) */
int dc_vertex_coords(const dc_model* model, double* coords, size_t n);
/* Dirichlet constraints from constrain.{boundary,skeleton}.expression (replaces the
 * constraints container filled by model/constraints.hh:51-199): *n_out receives their
 * number; with dofs / values non-null (n == *n_out) the constrained reference DOF indices
 * (ascending in the engine's blocked order) and their values are copied out. */
int dc_constraints(const dc_model* model, int64_t* dofs, double* values, size_t n, size_t* n_out);

/* Replaces make_initial + interpolate (dune/copasi/model/make_initial.hh:24-90,
 * interpolate.hh:21-78): nodal interpolation of initial.expression at time_begin. */
int dc_state_set_initial(dc_model* model);
/* full coefficient vector in the reference DOF order (State::coefficients,
 * model/model.hh:36-42): compartment-major, vertex-major, species interleaved */
int dc_state_get(const dc_model* model, double* host_out, size_t n);
int dc_state_set(dc_model* model, const double* host_in, size_t n, double time);

/* VTK output of the current state (replaces Model::write_vtk, dune/copasi/model/model.hh:88,
 * model_multi_compartment.impl.hh:219-293, driven by writer.vtk.path in the reference CLI):
 * per compartment "<path>/<stem>-<compartment>-NNNNN.vtu" (stem = last component of path,
 * NNNNN = call index for this path) with one vertex field per species, and the time series
 * "<path>/<stem>-<compartment>.pvd".  append = 0 starts a new series. */
int dc_write_vtk(const dc_model* model, const char* path, int append);
int dc_state_get_species(const dc_model* model, int32_t species, double* host_out, size_t n);
int dc_state_time(const dc_model* model, double* time);

/* Replaces SimpleAdaptiveStepper::do_step (dune/copasi/common/stepper.hh:337-368):
 * one step with dt, halving on failure down to time_step_min; on success *dt becomes
 * the suggested next step (x increase factor, clamped to time_step_max). */
int dc_step(dc_model* model, double* dt, dc_step_info* info);
/* Replaces TimeStepper::evolve + snap_to_time (stepper.hh:144-239): steps until t_end,
 * calling `cb` after every successful step. */
int dc_evolve(dc_model* model, double t_end, double* dt, dc_callback cb, void* user);

/* Operator entry points (the local-operator boundary, local_operator.hh:417-707 and
 * :777-1203, as driven by PDELab's instationary assembler): at state x (reference
 * order) and time t, r = cm * M(x) + ca * A(x) and the BSR values of
 * cm * dM/dx + ca * dA/dx.  r and jac_values may be NULL. */
int dc_assemble(dc_model* model, const double* x, double t, double cm, double ca, double* r, double* jac_values,
                size_t n_jac_values);
/* Matrix-free Jacobian product (replaces the local operators' jacobian_apply,
 * local_operator.hh:510-524, 1354-1396, 1438-1455, as driven by
 * PDELab::makeInstationaryMatrixFreeAssembler, make_step_operator.hh:289-293): at state x and
 * time t, y = (cm * dM/dx + ca * dA/dx) v with every state-dependent volume and face term
 * evaluated per element / face (vectors in reference order, ndof entries).  The Newton
 * solve uses the same product under linear_solver.matrix_free = true. */
int dc_jacobian_apply(dc_model* model, const double* x, double t, double cm, double ca, const double* v, double* y);
/* No counterpart in the reference.  Residual assembly that allocates nothing, for callers
 * that cannot allocate device memory when they need a residual (their device memory is
 * owned by another allocator, or cudaMalloc/cudaFree would synchronise the device inside a
 * latency-bound loop).  Same result as dc_assemble(model, x, t, cm, ca, r, NULL, 0), with
 * x and r host arrays in the reference DOF order.  The state and residual are staged in a
 * fixed 16 MiB device array compiled into the library, held by every GPU that loads it:
 * models with more than 2^20 DOF, or whose compartments carry different species counts,
 * return DC_ERR_ARGUMENT.  All calls on a device share the array; calls that overlap on
 * the GPU race.  The call runs on the model's device whatever device is current.
 * dc_model_create looks up the array's address on the model's device, which loads the
 * module holding the array and commits it there; should that lookup fail, the first call
 * retries it, so create the model (or make one call) before any stream capture.  x and r
 * hold n_dof doubles each.  Returns a status code only (DC_ERR_CUDA for a CUDA failure);
 * dc_last_error() is not updated. */
int dc_assemble_residual_noalloc(dc_model* model, const double* x, double t, double cm, double ca, double* r);

/* BSR pattern of the Jacobian (block rows = (compartment, vertex) pairs) */
int dc_pattern(const dc_model* model, int32_t* rowptr, size_t n_rowptr, int32_t* colidx, size_t n_colidx);
/* map from reference DOF index to padded device index (node * block_size + species) */
int dc_dof_map(const dc_model* model, int64_t* ref_to_dev, size_t n);

/* Newton iterations of every stage solve of the last dc_step, in stage order (stages of
 * attempts that the stepper rejected first, then the accepted attempt's stages; a stage
 * whose Newton solve failed adds no entry; linear models add none).  Replaces reading
 * PDELab's NewtonOperator result per stage (the Newton of model/make_step_operator.hh:
 * 246-288, run by the RungeKutta one-step method once per stage, :408-443).  *n_out
 * receives the count; with counts non-null (n >= *n_out) the values are copied. */
int dc_step_stage_newton(const dc_model* model, int32_t* counts, size_t n, size_t* n_out);

/* solver statistics accumulated since creation */
int dc_stats(const dc_model* model, int64_t* newton_iterations, int64_t* linear_iterations, int64_t* assemblies,
             int64_t* failed_steps);

/* set the linear-solve precision: 0 = fp64 BiCGSTAB, 1 = fp32 BiCGSTAB inside fp64 iterative refinement */
int dc_set_mixed_precision(dc_model* model, int enabled);

/* Replaces the parser interface (dune/copasi/parser/parser.hh:15-62: define_variable,
 * set_expression, compile, operator()) for host-side checks: compiles `expression` with
 * the parser_context section of `context_ini` (may be NULL) and the n variables
 * names[i] = values[i], evaluates it on the host and writes the value to *out.  No GPU
 * is needed. */
int dc_expr_eval(const char* expression, const char* context_ini, const char* const* names, const double* values,
                 int32_t n, double* out);

/* Instrumentation (no reference counterpart; replaces the reference's perfetto trace
 * counters of LinearSolver / TimeStep, model/make_step_operator.hh:104-139):
 * the CUDA stream the model launches on (cudaStream_t as void*), the number of kernels
 * this library has launched, and per-category device times measured with CUDA events
 * (0 = residual-only assembly passes, 1 = SpMV, 2 = preconditioner apply, 3 = single-launch
 * BiCGSTAB solves, whose call count is the number of Krylov iterations they ran,
 * 4 = Jacobian-only assembly passes, 5 = combined residual + Jacobian assembly passes)
 * while profiling is enabled. */
int dc_stream_handle(const dc_model* model, void** stream);
int64_t dc_launch_count(void);

/* Self-test of the bounded device waits (no reference counterpart): runs one grid-wide
 * barrier of the single-launch solve's kind that cannot complete (4 cooperative blocks, 50 ms
 * limit).  Every block's wait must give up and flag it; *gave_up_blocks receives how many did
 * and *elapsed_ms the kernel's duration.  The CUDA context stays usable afterwards. */
int dc_selftest_barrier_timeout(double* gave_up_blocks, double* elapsed_ms);
/* Run-time compilation self-test (no reference counterpart; needs no GPU): generates the
 * volume kernels of a synthetic two-species compartment whose terms cover every volume term
 * kind, in 2D and 3D, and compiles them with NVRTC for sm_103a.  Returns DC_OK, or
 * DC_ERR_CONFIG with the reason in `message` (NVRTC missing, compilation log). */
int dc_jit_selftest(char* message, size_t len);
/* Volume kernels of the model (no reference counterpart): copies "compiled" (kernels
 * compiled at set-up for the model's expression programs), "off" (the bytecode
 * interpreter kernels) or "interpreter (<reason>)" into buf.  Set by model.assembly.jit =
 * auto | true | false (auto: compiled for compartments of at least 2^18 cells). */
int dc_model_jit_status(const dc_model* model, char* buf, size_t len);
/* Preconditioner of the model's linear solves (no reference counterpart; the reference logs
 * "Creating preconditioner with type ...", preconditioner.hh:127-128): a JSON object with the
 * type and its structure (colours of the multicolour sweeps; rows, blocks and kernel kind per
 * multigrid level), copied into buf. */
int dc_precond_info(const dc_model* model, char* buf, size_t len);
/* Arithmetic throughput of the current device (no reference counterpart; instrumentation
 * for the roofline of the FP64-bound assembly): FP64 and FP32 fused multiply-add rates in
 * TFLOP/s (2 flops per FMA), measured with independent FMA chains on every SM (~20 ms). */
int dc_selftest_fma_peaks(double* fp64_tflops, double* fp32_tflops);
/* Preconditioner building blocks on a caller-given block matrix (no reference counterpart;
 * test instrumentation of the preconditioners that replace dune-istl's SeqSSOR / SeqSOR /
 * SeqILU / SeqDILU, dune/copasi/solver/istl/factory/preconditioner.hh:94-112, and of the
 * engine's multigrid).  Graphs are CSR on the host (nrows rows, rowptr[nrows] entries,
 * self-loops allowed).
 * dc_selftest_color: the colouring the multicolour preconditioners use (colour_out[nrows],
 * *ncolours).  dc_selftest_aggregate: the multigrid's aggregation of one level (rows of
 * different group, NULL: one group, never share an aggregate; distance 1 or 2) into
 * agg_out[nrows], *naggregates.  dc_selftest_precond: builds preconditioner `kind` ("SSOR",
 * "SOR", "ILU", "DILU" or "AMG") for the BSR matrix (block size bs, row-major blocks in
 * vals, every row holding its diagonal block), with `params` "key=value;..." (relaxation,
 * iterations; AMG: smoother 0 Jacobi / 1 L1-Jacobi / 2 Gauss-Seidel / 3 ILU(0), relaxation,
 * coarse_sweeps, max_level, coarsen_target, aggregation_distance, coarse_correction,
 * warp_rows_below, finest_post_smoothing, w_levels), applies it once to r
 * (in fp64, or in fp32 when fp32 != 0) and writes z (nrows * bs).  info (8 doubles, may be
 * NULL): colours, or for AMG the levels, the dense coarse solve's unknowns (0: none) and
 * the rows of levels 0 to 5. */
int dc_selftest_color(int64_t nrows, const int32_t* rowptr, const int32_t* colidx, int32_t* colour_out,
                      int32_t* ncolours);
int dc_selftest_aggregate(int64_t nrows, const int32_t* rowptr, const int32_t* colidx, const int32_t* group,
                          int32_t distance, int32_t* agg_out, int64_t* naggregates);
int dc_selftest_precond(const char* kind, const char* params, int64_t nrows, int32_t bs, const int32_t* rowptr,
                        const int32_t* colidx, const double* vals, const int32_t* group, const double* r, double* z,
                        int32_t fp32, double* info);
int dc_profile_enable(dc_model* model, int enabled);
int dc_profile_get(const dc_model* model, double* ms, int64_t* calls, int32_t n_categories);

/* Transform/reduce operators on the current state (replaces Model::reduce,
 * dune/copasi/model/model.hh:24-101, implemented in model/diffusion_reaction/reduce.hh:40-285).
 * reduce_ini: ini text holding a [model.reduce] section or the section's keys at top level
 * ("mass.evaluation.expression = u*integration_factor" ...); NULL uses the model's own
 * [model.reduce].  *n_out receives the number of keys; with out non-null (n >= *n_out) the
 * results are written in key order.  A key whose error.expression evaluates non-zero has
 * error = 1 (the reference then throws ReductionError); warn likewise for warn.expression. */
typedef struct dc_reduce_value {
  char key[64];
  double value;
  int32_t error;
  int32_t warn;
} dc_reduce_value;
int dc_reduce(const dc_model* model, const char* reduce_ini, dc_reduce_value* out, size_t n, size_t* n_out);

/* Layout of the single-precision Krylov operator (no reference counterpart): -1 = not yet
 * chosen, 0 = BSR with a thread per scalar row, 1 = SELL-32 with a warp per 32 block rows.
 * `linear_solver.spmv = auto` (default) times both on the first fp32 operator and keeps the
 * faster; bsr_us / sell_us receive those times in microseconds (0 when not tuned). */
int dc_spmv_format(const dc_model* model, int32_t* format, double* bsr_us, double* sell_us);

/* Request server (no counterpart in the reference, which runs one simulation per
 * process): simulations are submitted as INI text (+ optional initial state in the
 * reference DOF order) and admitted as soon as their estimated device footprint fits
 * into `budget_bytes` and one of `max_active` slots is free; admitted requests run
 * concurrently, each on its own stream, and every result equals the same request run
 * alone.  The server handle is internally synchronised. */
typedef struct dc_server dc_server;

typedef struct dc_result {
  int64_t request_id;
  int32_t status;       /* DC_OK or the failing status */
  int32_t reserved;
  double queue_s;       /* submit -> admission */
  double run_s;         /* admission -> completion */
  double latency_s;     /* submit -> completion */
  int64_t n_dof;
  int64_t newton_iterations;
  int64_t linear_iterations;
  int64_t steps;
  int64_t bytes_estimate;  /* footprint estimated at submission (admission charge) */
  int64_t bytes_measured;  /* peak device bytes the simulation's buffers held; the server
                              charges a running simulation this instead of the estimate */
  double setup_s;          /* model and solver set-up, part of run_s */
} dc_result;

int dc_server_create(int64_t budget_bytes, int32_t max_active, dc_server** out);
/* dc_server_create with flags.  DC_SERVER_BATCH_KRYLOV: continuous batching of the running
 * simulations' block-Jacobi BiCGSTAB solves (fp64 solves and the fp32 corrections of the
 * mixed path): every such solve joins one batch whose five phase kernels walk a table of
 * 256-row tiles of all instances, replayed from captured CUDA graphs of 2, 4 or 8
 * iterations; instances join and leave between replays.  Results do not depend on the mix (per-instance
 * sums in a fixed order), but differ in rounding from the unbatched server's.  Other Krylov
 * methods and preconditioners stay on the simulation's own stream.  No counterpart in the
 * reference (one simulation per process; its LinearSolver solves one system at a time,
 * dune/copasi/model/make_step_operator.hh:102-146). */
#define DC_SERVER_BATCH_KRYLOV 1
int dc_server_create_ex(int64_t budget_bytes, int32_t max_active, int32_t flags, dc_server** out);
typedef struct dc_batch_stats {
  int64_t solves;        /* systems the batch solved */
  int64_t replays;       /* graph replays (2, 4 or 8 iterations of every active instance each) */
  int64_t slot_replays;  /* sum over replays of the instances active in them */
  int64_t iterations;    /* BiCGSTAB iterations of all solved systems */
  int32_t max_active;    /* most instances in one replay */
  int32_t reserved;
  double replay_s;       /* host time from the start of each replay to its end, summed */
  double wait_s;         /* time the simulations spent waiting for their solves, summed */
} dc_batch_stats;
/* counters of the Krylov batch (all zero for a server created without the flag) */
int dc_server_batch_stats(const dc_server* server, dc_batch_stats* out);
/* the batch's launch-shape autotuner: per precision, the replay grid (blocks) it settled on
 * for each batch size bucket, as JSON {"fp32": {"<tiles>": blocks, ...}, "fp64": {...}}
 * ("{}" for a server created without the flag) */
int dc_server_batch_tuning(const dc_server* server, char* buf, size_t len);
int dc_server_submit(dc_server* server, const char* ini_text, const char* overrides, const double* init_state,
                     size_t n_init, int64_t* request_id);
/* completed results, up to max; wait != 0 blocks until one is available (or none pending) */
int dc_server_poll(dc_server* server, int32_t wait, dc_result* results, int32_t max, int32_t* n_out);
/* final state of a completed request (reference DOF order); the server then drops it */
int dc_server_take_state(dc_server* server, int64_t request_id, double* host_out, size_t n);
/* footprint estimate used for admission (host only, no GPU needed) */
int dc_server_estimate(const char* ini_text, const char* overrides, int64_t* bytes);
/* waits for every submitted request, then frees the server */
int dc_server_destroy(dc_server* server);

/* message of the last failure on this thread ("" if none) */
const char* dc_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* DCGPU_H */
