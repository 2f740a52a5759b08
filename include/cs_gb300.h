/*
 * cs_gb300.h — C ABI of the GB300-native collocation solver (libcs_gb300.so).
 *
 * Solves the BVP-DAEs that the Pontryagin conditions of a nonlinear optimal
 * control problem give, y' = f(y,z,p), 0 = g(y,z,p,alpha), r(y(t0),y(tf),p)
 * = 0, by Lobatto IIIA collocation and a damped Newton method with mesh
 * refinement: the Newton inner loop of UW-OCP/Collocation-Solver-CUDA,
 * re-designed for one GB300 (sm_103a), FP64, with many instances per launch.
 *
 * The reference has no FFI: its boundary is a set of Python stage functions
 * that take numpy arrays and allocate device memory per call.  Each entry
 * point below names the reference function(s) it replaces
 * (collocation_solver_parallel_2d_shared.py = CS, solve_babd_system.py = SB).
 *
 * Conventions: every function returns CS_OK (0) or an error code and never
 * throws; cs_last_error() gives the message of the calling thread's last
 * error.  Host arrays are packed per instance in instance order: for node
 * arrays, instance b's rows start after the sum of N[0..b-1] rows.  One batch
 * is used by one host thread at a time; calls are ordered on the batch's
 * stream and return after it has finished.
 */
#ifndef CS_GB300_H
#define CS_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CS_OK 0
#define CS_ERR_INVALID 1   /* bad argument or size */
#define CS_ERR_CUDA 2      /* CUDA runtime/driver failure */
#define CS_ERR_NVRTC 3     /* run-time compilation of the problem failed */
#define CS_ERR_NOMEM 4     /* device allocation failed */
#define CS_ERR_STATE 5     /* call not valid in the batch's current state */

/* per-instance status after cs_solve (matches the device state machine) */
#define CS_STATUS_DONE 3
#define CS_STATUS_FAIL 4
/* spare instance not started (holds its initial guess), and spare stopped
 * because its primary succeeded (its state is then undefined); see
 * cs_batch_set_spares */
#define CS_STATUS_PARKED 6
#define CS_STATUS_CANCELLED 7

typedef struct cs_module cs_module;
typedef struct cs_batch cs_batch;

/* A compiled problem for one number of collocation points m.  problem_src
 * holds the CUDA device functions cs_f, cs_g, cs_Df, cs_Dg, cs_r, cs_Dr
 * (emitted from the OCP derivation); the tables are the Lobatto IIIA tableau
 * and the mesh-error quadrature for this m.
 * Replaces: the numba JIT of the generated bvp_problem.py functions
 * (OCP2ABVP.py:203-327) and of every CS/SB kernel. */
typedef struct cs_module_desc {
  const char* problem_src;
  int ny, nz, np;       /* sizes of y, z, p */
  int np_eff;           /* leading parameters that f, g depend on */
  int n_theta;          /* instance constants */
  int m;                /* collocation points, 2..10 */
  const double* lobatto_A;  /* m*m */
  const double* lobatto_b;  /* m */
  const double* lobatto_c;  /* m */
  const double* gauss_w;    /* m+1 */
  const double* gauss_L;    /* (m+1)*m: L_k at the Gauss points */
  const double* gauss_I;    /* (m+1)*m: integral of L_k at the Gauss points */
  const double* L0;         /* m: L_k(0) */
  const double* L1;         /* m: L_k(1) */
  const char* cache_dir;    /* compiled-code cache directory, or NULL */
  int layout;               /* 0: automatic; 1: stage systems and BABD blocks in
                               shared memory (fails if they do not fit);
                               2: large-system kernels (global-memory slab per
                               CTA, blocked LU), chosen automatically when the
                               blocks do not fit in shared memory */
  int precision;            /* large-system condensation: 0 FP64; 1 TF32,
                               2 BF16 tensor cores with FP32 storage and
                               accumulation (an inexact Newton Jacobian: the
                               residual, line search, mesh error and BABD
                               solve stay FP64); 3 / 4: TF32 / BF16 also for
                               the tree merges' block updates (their rounding
                               compounds over the tree's levels; cs_opts.refine
                               sweeps of FP64 iterative refinement correct each
                               Newton direction).  Nonzero implies the
                               large-system condensation. */
} cs_module_desc;

/* Compile (or load from the cache) and load the module on the current device. */
int cs_module_load(const cs_module_desc* desc, cs_module** out);
void cs_module_free(cs_module* mod);

/* Solver options; the defaults (cs_opts_default) are the reference's
 * (CS:58-76): alpha0 = 0.1, beta = 0.9, 20 line-search halvings, min 3 nodes. */
typedef struct cs_opts {
  double tol;            /* BvpDae.tolerance */
  int max_iter;          /* BvpDae.maximum_newton_iterations */
  int max_mesh;          /* BvpDae.maximum_mesh_refinements */
  int max_nodes;         /* BvpDae.maximum_nodes */
  int min_nodes;
  int max_linesearch;
  double alpha0;         /* initial continuation parameter */
  double alpha_m;        /* final continuation parameter (0.1, or 1e-6 with inequalities) */
  double beta;           /* continuation factor */
  int check_every;       /* Newton super-steps between host checks for completion */
  int babd_path;         /* Newton direction kernels: 0 automatic (one launch per tree
                            level, the top 4 levels and the top system in one CTA per
                            instance where the block rows allow), 1 one CTA per instance
                            for everything, 2 one launch per tree level and for the top */
  int residual_type;     /* segment residual estimate (CS:29-32): 1 weighted sum
                            (default), 2 weighted squares, 0 weighted maximum */
  int scale_by_time;     /* multiply the running estimate by h (default 1) */
  int residual2;         /* 1: the residual2 estimate instead (CS:1895-2013) */
  int refine;            /* tree merges on the tensor cores (precision 3, 4): sweeps of
                            FP64 iterative refinement of every Newton direction (the
                            residual of the condensed system in FP64, a correction from
                            the same tree); default 2, 0 off.  No reference counterpart
                            (the reference solves in FP64 only) */
  int ls_grow;           /* speculative line search: after a search that rejected k trials,
                            the next one evaluates min(20, ls_grow * k + 2) trials in its
                            first super-step (the rest, if needed, in the next); default 2,
                            0: all 20.  The trials are taken in the reference's order
                            (CS:155-174), so results and counts do not depend on it */
} cs_opts;

void cs_opts_default(cs_opts* o);

/* Options the stage entry points use (cs_solve sets its own from its
 * argument): the segment residual estimate of cs_stage_segment_residual and
 * the line-search / continuation constants.  No reference counterpart (the
 * reference reads module globals). */
int cs_batch_set_opts(cs_batch* bt, const cs_opts* opts);

/* Per-instance counters after a solve (the reference's benchmark counts). */
typedef struct cs_stats {
  int status;            /* CS_STATUS_DONE or CS_STATUS_FAIL */
  int N;                 /* final number of nodes */
  int newton_steps;      /* Jacobian evaluations ("Jacobian counts") */
  int residual_evals;    /* "Residual counts" */
  int segment_evals;     /* "Segment Residual counts" */
  int remeshes;
  int continuation_steps;
  int singular;          /* singular pivots met */
  int fail_reason;       /* 0 none, 1 Newton/continuation iteration limit,
                            2 node count outside [min, max], 3 mesh limit */
  double alpha;          /* final continuation parameter */
  double max_residual;   /* last maximum segment residual */
  double last_norm;      /* last residual infinity norm */
} cs_stats;

/* Device workspace for `batch` instances and up to node_capacity node slots
 * in total (grown on demand by remeshing).  stream: a cudaStream_t, or NULL
 * for a new stream owned by the batch. */
int cs_batch_create(cs_module* mod, int batch, long long node_capacity, void* stream, cs_batch** out);
void cs_batch_free(cs_batch* bt);

/* Initial guess from HOST arrays: N[b] nodes, t (sum N), y (sum N x ny),
 * z (sum N x nz) at the nodes, p (batch x np), theta (batch x n_theta, may be
 * NULL when n_theta = 0); then forms the stage values (y' = f at the linearly
 * interpolated stage points).
 * Replaces: BvpDae.T0/Y0/Z0/P0 + form_initial_input_parallel (CS:287-356). */
int cs_batch_set_guess(cs_batch* bt, const int* N, const double* t, const double* y, const double* z,
                       const double* p, const double* theta);

/* Full iterate from HOST arrays: nodes as in cs_batch_set_guess, and the
 * stage values ydot ((N[b]-1) x m x ny per instance, packed) and zt
 * ((N[b]-1) x m x nz per instance, packed), used as they are.
 * Replaces: the (y, y_dot, z_tilde, p) arguments the reference passes to each
 * stage function (e.g. compute_f_q_parallel, CS:399). */
int cs_batch_set_state(cs_batch* bt, const int* N, const double* t, const double* y, const double* ydot,
                       const double* zt, const double* p, const double* theta);

/* Full solve of every instance: continuation, Newton with line search,
 * segment residual, remesh.
 * Replaces: collocation_solver_parallel (CS:36-251). */
int cs_solve(cs_batch* bt, const cs_opts* opts);

/* Progress hook of cs_solve: called on the solving thread after every check
 * of the Newton phase (every opts.check_every super-steps), with the number of
 * instances still in the Newton iteration and the super-steps run so far in
 * this solve.  The batch's stream is idle during the call, so the hook may
 * read the batch (cs_get_solution with null arrays returns the statuses); it
 * must not launch work on it.  fn = NULL removes the hook.  No counterpart in
 * the reference, which prints its progress (CS:60-251). */
typedef void (*cs_progress_fn)(void* user, int active, long long super_steps);
int cs_batch_set_progress(cs_batch* bt, cs_progress_fn fn, void* user);

/* Current node counts (batch ints) and total node slots. */
int cs_batch_sizes(cs_batch* bt, int* N_out, long long* total_out);

/* Solution to HOST arrays sized by the current node counts (z recovered at the
 * nodes); any pointer may be NULL.  stats: batch entries or NULL.
 * Replaces: recover_solution_parallel (CS:2034-2075) and the arrays handed to
 * bvpdae_write_data (CS:233-237). */
int cs_get_solution(cs_batch* bt, double* t, double* y, double* z, double* p, cs_stats* stats);

/* ---- stage entry points (one stage on the current iterate; host outputs) ---- */

/* Residual at the current iterate: per-instance infinity norm; optionally the
 * pieces f_a (slots x m(ny+nz)) and f_b (slots x ny), slot = node slot of the
 * interval's left node.
 * Replaces: compute_f_q_parallel (CS:399-512) + np.linalg.norm (CS:116). */
int cs_stage_residual(cs_batch* bt, double alpha, double* norms, double* f_a, double* f_b);

/* Newton direction at the current iterate: condensed blocks (slots x
 * ny*(2ny+np_eff+1): A | C | H | b column-major, may be NULL), dy (nodes x
 * ny), dydot (slots x m x ny), dzt (slots x m x nz), dp (batch x np).
 * Replaces: construct_jacobian_parallel, reduce_jacobian_parallel (CS:611-1001),
 * SB.partition_factorization_parallel, construct_babd_mshoot, qr_decomposition,
 * backward_substitution, partition_backward_substitution_parallel (SB:93-572),
 * recover_delta_k_parallel (CS:1580-1650). */
int cs_stage_newton_direction(cs_batch* bt, double alpha, double* rows, double* dy, double* dydot, double* dzt,
                              double* dp);

/* Segment residual per node slot (interval residual / tol; the last node of
 * each instance holds |r|_inf / tol) and the per-instance maximum.
 * Replaces: compute_segment_residual_parallel (CS:1770-1892). */
int cs_stage_segment_residual(cs_batch* bt, double alpha, double tol, double* res, double* max_res);

/* Remesh every instance with the given per-node residuals (host, node
 * slots), then re-form the stage values; N_new receives the new node counts.
 * Replaces: recover_solution_parallel + remesh + form_initial_input_parallel
 * (CS:194-198, 2034-2311). */
int cs_stage_remesh(cs_batch* bt, const double* res, int* N_new);

/* Solve one BABD system (the linear system of a Newton step after
 * condensation) given in DEVICE memory, reference layout (row-major):
 *   A, C: n x ny x ny;  H: n x ny x np;  b: n x ny      (block rows i = 0..n-1:
 *   A_i dy_i + C_i dy_{i+1} + H_i dp = b_i)
 *   B0, Bn: (ny+np) x ny;  Vn: (ny+np) x np;  r: ny+np   (B0 dy_0 + Bn dy_n +
 *   Vn dp = -r)
 * Outputs dy ((n+1) x ny) and dp (np) in device memory; *singular (host, may
 * be NULL) is set when the top system was singular (dy_0, dy_n, dp are then 0,
 * as the reference's LinAlgError fallback).  1 <= ny <= 32, 0 <= np <= 32.
 * Allocates its scratch (about 8 (2 ny (2ny+np+1) + ny (3ny+np+1)) bytes per
 * interval) for the duration of the call; ordered on `stream` (a
 * cudaStream_t or NULL) and returns after it has finished.
 * Replaces: partition_factorization_parallel, construct_babd_mshoot,
 * qr_decomposition, backward_substitution, recover_babd_solution and
 * partition_backward_substitution_parallel (solve_babd_system.py:93-572). */
int cs_babd_solve(int ny, int np, int n, const double* A, const double* C, const double* H, const double* b,
                  const double* B0, const double* Bn, const double* Vn, const double* r, double* dy, double* dp,
                  int* singular, void* stream);

/* cs_babd_solve without any device allocation, for callers that cannot call
 * cudaMalloc: code that runs inside a memory pool or allocator it must not
 * re-enter, or under a framework that owns all device memory.  It has no counterpart in the reference (whose stage
 * functions allocate device arrays on every call).
 * Same arguments and results as cs_babd_solve.  Its scratch is a fixed 32 MiB
 * array compiled into this library, held by every GPU that loads the library
 * until the process exits; systems needing more (2 n ny (2ny+np+1) +
 * (n+1) ny (3ny+np+1) doubles, plus 256 bytes) are rejected with
 * CS_ERR_INVALID.  The first call on each device looks up the array's device
 * address (cudaGetSymbolAddress); make that first call before any stream
 * capture.  All calls share the one array: calls that overlap on the GPU
 * (other streams, other host threads) race and must be serialised by the
 * caller. */
int cs_babd_solve_noalloc(int ny, int np, int n, const double* A, const double* C, const double* H,
                          const double* b, const double* B0, const double* Bn, const double* Vn, const double* r,
                          double* dy, double* dp, int* singular, void* stream);

/* The tensor-core block update C -= A B^T on one matrix in DEVICE memory:
 * C (M x N, FP32, row stride ldc), A (M x K, row stride lda) and B (N x K, row
 * stride ldb) in FP32, rounded to TF32 (precision 1, round to nearest, ties
 * away) or BF16 (precision 2, round to nearest even) on the tensor cores
 * (tcgen05.mma, FP32 accumulation in tensor memory).  1 <= M <= 256,
 * 1 <= N <= 512, 1 <= K <= 64; ordered on `stream` and returns after it has
 * finished.  It is the trailing update of the reduced-precision blocked LU
 * that condenses large stage systems (the LU of
 * collocation_solver_parallel_2d_shared.py:887-1001 and
 * matrix_factorization_cuda.py:91-165, there in FP64 without tensor cores),
 * exposed on its own so that the update can be checked and used alone. */
int cs_tc_update(int precision, int M, int N, int K, const float* A, int lda, const float* B, int ldb, float* C,
                 int ldc, void* stream);

/* The solution file of every instance in the reference's text format
 * (BVPDAEReadWriteData: labels, then t, y and z rows and p, every number as
 * Python's "{}".format of the double prints it), formatted on the GPU from
 * the values cs_get_solution returns.  offsets (B + 1 entries) are always
 * filled: file b is out[offsets[b] .. offsets[b+1]).  out = NULL only sizes
 * the files; a cap below offsets[B] fails with CS_ERR_INVALID.
 * Replaces: the per-value Python writer (BVPDAEReadWriteData.py:337-364)
 * called once per solution. */
int cs_format_solutions(cs_batch* bt, char* out, long long cap, long long* offsets);

/* One double as that text ("{}".format / repr: shortest round-trip digits),
 * host code: out needs 25 bytes; returns the length (-1: out is NULL). */
int cs_format_double(double v, char* out);

/* Current iterate to host: t, y (nodes), ydot, z~ (slots), z at nodes, p. */
int cs_get_state(cs_batch* bt, double* t, double* y, double* ydot, double* zt, double* z_nodes, double* p);

/* Restore the initial guess given to the last cs_batch_set_guess from its
 * device copy (no host transfer) and re-form the stage values: lets a caller
 * re-solve the same batch with inputs already resident in HBM. */
int cs_batch_reset(cs_batch* bt);

/* Work and timing counters of a batch since the last cs_profile_reset.
 * With timing on, the condensation, BABD and residual launches are bracketed
 * by CUDA events on the batch's stream. */
typedef struct cs_profile {
  long long launches;             /* kernel launches issued by the library */
  long long super_steps;          /* Newton super-steps */
  long long intervals_condensed;  /* interval condensations (units of k_condense) */
  long long systems_solved;       /* BABD solves (units of k_babd) */
  long long residual_intervals;   /* interval residual evaluations */
  long long condense_launches, babd_launches, residual_launches;
  double condense_ms, babd_ms, residual_ms;  /* summed event times (timing on) */
} cs_profile;

int cs_profile_reset(cs_batch* bt, int timing);
int cs_profile_get(cs_batch* bt, cs_profile* out);

/* Page-locked host memory for the host arrays of the calls above. */
void* cs_pinned_alloc(size_t bytes);
void cs_pinned_free(void* p);

/* ---- learned warm start: a multilayer perceptron trained on solutions ----
 * depth linear layers n_in -> width -> ... -> width -> n_out, GELU between
 * them; FP32 master weights, BF16 operands with FP32 accumulation on the
 * tensor cores, MSE loss on normalised outputs, Adam.  Host arrays are
 * row-major float32 (one row per sample).  No counterpart in the reference
 * (its Newton starts from the OCP file's constant estimates). */
typedef struct cs_mlp cs_mlp;
int cs_mlp_create(int n_in, int width, int depth, int n_out, unsigned long long seed, cs_mlp** out);
void cs_mlp_free(cs_mlp* mlp);
long long cs_mlp_num_params(const cs_mlp* mlp);
/* inputs and outputs are normalised as (v - mean) / std inside the network */
int cs_mlp_set_normalization(cs_mlp* mlp, const float* in_mean, const float* in_std, const float* out_mean,
                             const float* out_std);
/* all weights and biases, layer by layer (W[out][in] then b[out]) */
int cs_mlp_get_params(cs_mlp* mlp, float* host);
int cs_mlp_set_params(cs_mlp* mlp, const float* host);
/* mean-squared error (normalised outputs) of n samples and its gradient */
int cs_mlp_gradient(cs_mlp* mlp, const float* X, const float* Y, int n, double* loss, float* grad);
int cs_mlp_train(cs_mlp* mlp, const float* X, const float* Y, int n, int epochs, int batch, float lr,
                 unsigned long long seed, double* final_loss);
/* learning-rate schedule of cs_mlp_train: lr_final >= 0 decays the rate of
 * every call along a half cosine from lr to lr_final * lr over the call's
 * steps; lr_final < 0 (the default) keeps it constant */
int cs_mlp_set_schedule(cs_mlp* mlp, float lr_final);
int cs_mlp_predict(cs_mlp* mlp, const float* X, int n, float* Y);

/* forward pass on DEVICE arrays (n rows), ordered on `stream` (cudaStream_t
 * or NULL); returns after the stream has finished */
int cs_mlp_predict_device(cs_mlp* mlp, const float* dX, int n, float* dY, void* stream);

/* Warm start of a batch from per-instance trajectory vectors in DEVICE
 * memory: row b (stride floats) holds y and z at n_nodes equispaced
 * normalised times in [0, 1] (node-major: n_nodes x ny, then n_nodes x nz)
 * followed by p.  For every instance, y and z at its current mesh nodes are
 * interpolated linearly in (t - t_0) / (t_N - t_0), p is taken over, the stage
 * values are re-formed and the instance restarts from Newton (continuation
 * parameter alpha0).  Replaces the constant estimates of the OCP file
 * (OCP2ABVP.py:402-447) as the Newton initial guess; no reference
 * counterpart. */
int cs_batch_warm_start(cs_batch* bt, int n_nodes, const float* traj, int stride);

/* Fallback inside the batch.  With n_primary > 0 the batch (B = 2 n_primary
 * instances) pairs instance k < n_primary, the primary, with instance
 * n_primary + k, its spare: the same problem instance from another initial
 * guess (normally the plain one, with the primary warm-started).  Spares are
 * parked (CS_STATUS_PARKED, untouched by every kernel) by cs_batch_set_guess,
 * cs_batch_set_state and cs_batch_reset, and by this call when it changes the
 * pairing (the spares not started since their guess was set); and
 * cs_batch_warm_start fills only the primaries (traj holds n_primary rows).
 * During cs_solve, once at most `trigger` instances are in the Newton
 * iteration, the spare of every primary still iterating or failed starts from
 * its initial guess in the same super-steps as the rest of the batch, and a
 * spare whose primary has succeeded is stopped (CS_STATUS_CANCELLED); before
 * cs_solve returns, the spare of every failed primary has run.  A started
 * spare's result is the one of solving it alone from its initial guess, so a
 * primary that fails takes its spare's solution: the outcome of solving the
 * failed instances again afterwards, in one pass.  trigger < 0 keeps the
 * spares parked; n_primary = 0 removes the pairing (instances parked stay so
 * until the next set_guess / reset).  No reference counterpart (the reference
 * solves one initial guess per call, CS:36-251). */
int cs_batch_set_spares(cs_batch* bt, int n_primary, int trigger);

/* Device memory for callers of the device-pointer entry points. */
void* cs_device_alloc(size_t bytes);
void cs_device_free(void* p);
/* kind: 0 host to device, 1 device to host, 2 device to device; synchronous */
int cs_copy(void* dst, const void* src, size_t bytes, int kind);

/* Message of this thread's last error ("" if none). */
int cs_last_error(char* buf, size_t len);

/* Time one launch of the condensation kernel on the current iterate, in
 * milliseconds, with CUDA events on the batch's stream (for roofline figures). */
int cs_time_condense(cs_batch* bt, int reps, double* ms);

/* Launch-shape tuner of the condensation (the per-(m, ny) tile shape):
 * times every candidate on the batch's current intervals -- 4, 8, 16 or 32
 * lanes per interval x 1..8 warps per CTA for shared-memory stage systems,
 * 128 or 256 threads per CTA for the large-system kernel -- and makes the
 * fastest the module's shape for all its batches.  No reference
 * counterpart. */
typedef struct cs_tune_result {
  int lanes;          /* lanes per interval, 0: one CTA per interval */
  int block;          /* threads per CTA */
  int grid;           /* CTAs of the persistent grid */
  int candidates;     /* shapes timed */
  double ms;          /* one condensation of the batch, chosen shape */
  double default_ms;  /* ... with the shape chosen from occupancy rules */
} cs_tune_result;
int cs_autotune_condense(cs_batch* bt, int reps, cs_tune_result* out);

/* FP64 FMA throughput of this GPU, measured by a register-resident DFMA loop
 * (TFLOP/s, counting an FMA as 2 flops); the denominator of FP64 roofline
 * fractions. */
int cs_measure_fp64_peak(double* tflops);

/* FP64 throughput of the tensor cores (mma.sync m8n8k4 f64, "DMMA") in
 * TFLOP/s from a register-resident loop over the whole GPU, to compare with
 * cs_measure_fp64_peak (DFMA on the FP64 pipe).  No reference counterpart. */
int cs_measure_dmma_peak(double* tflops);

/* Start / stop the profiler's collection range (cudaProfilerStart/Stop), so
 * a profiler launched with collection off from the start captures exactly
 * the region between them.  No reference counterpart. */
int cs_profiler_start(void);
int cs_profiler_stop(void);

#ifdef __cplusplus
}
#endif

#endif /* CS_GB300_H */
