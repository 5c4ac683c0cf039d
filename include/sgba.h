/*
 * sgba.h -- C ABI of the GB300 Schur-complement Levenberg-Marquardt bundle
 * adjustment path (libsgba.so).
 *
 * This is the drop-in boundary for sophus-rs's
 *   optimize_nlls(variables, cost_fns, eq_fns, params)
 *     (crates/sophus_opt/src/nlls.rs:73-83)
 * and the stateful
 *   Optimizer::new / Optimizer::step / Optimizer::build_solution
 *     (crates/sophus_opt/src/nlls/optimizer.rs:71-120, 345-376, 609-646)
 * when the problem is the bundle-adjustment specialisation:
 *   - one CostFn of PinholeCameraReprojectionCostTerm
 *     (crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:28-95),
 *     optionally with RobustKernel::Huber (crates/sophus_opt/src/robust_kernel.rs);
 *   - families: intrinsics Conditioned, poses (Isometry3F64) Free with
 *     constant ids, points (VecF64<3>) Marginalized with constant ids;
 *   - params.solver = SchurBlockSparseLdlt (crates/sophus_solver/src/lib.rs:313).
 *
 * All pointers are plain host pointers; the library copies what it needs to
 * device memory.  Every function returns an sgba_status (0 = OK, negative =
 * error class mirroring NllsError, crates/sophus_opt/src/nlls/optimizer_types.rs:422-504);
 * sgba_last_error() returns the message of the calling thread's last error.
 * A problem handle is not thread-safe; it owns one CUDA stream.
 */
#ifndef SGBA_H
#define SGBA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SGBA_ABI_VERSION 2

typedef enum {
  SGBA_OK = 0,
  SGBA_ERR_INVALID_ARGUMENT = -1,     /* bad pointer, size, index or non-finite input */
  SGBA_ERR_INVALID_PARAMS = -2,       /* pose quaternion fails | |q| - 1 | <= 1e-6 (from_params) */
  SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG = -3, /* NllsError::SchurMissingFreeOrMarg */
  SGBA_ERR_UNSUPPORTED = -4,          /* configuration outside this path */
  SGBA_ERR_CUDA = -5,                 /* CUDA runtime failure (message has the CUDA error) */
  SGBA_ERR_OUT_OF_MEMORY = -6,
  SGBA_ERR_STATE = -7,                /* call out of order (e.g. step before init) */
  SGBA_ERR_DEVICE_TIMEOUT = -8,       /* a bounded device wait gave up */
  SGBA_ERR_FACTORIZATION = -9,        /* covariance: H_mm or S could not be factored */
} sgba_status;

/* Problem description (host SoA; the caller keeps ownership, the library copies).
 * Mirrors the VarBuilder families "cams" (Conditioned intrinsics), "poses"
 * (Free Isometry3F64 with const ids) and "points" (Marginalized VecF64<3>
 * with const ids) plus the CostTerms of PinholeCameraReprojectionCostTerm. */
typedef struct {
  int32_t n_cam;              /* number of poses */
  const double *poses;        /* n_cam*7: world_from_camera params (qw qx qy qz tx ty tz) */
  const uint8_t *pose_const;  /* n_cam flags (1 = constant id), or NULL */
  int32_t n_pt;
  const double *points;       /* n_pt*3 world points */
  const uint8_t *point_const; /* n_pt flags, or NULL */
  double intrinsics[4];       /* fx fy cx cy (PinholeCameraF64 params, Conditioned) */
  int64_t n_obs;
  const int32_t *obs_cam;     /* pose index per observation (entity_indices[1]) */
  const int32_t *obs_pt;      /* point index per observation (entity_indices[2]) */
  const double *obs_uv;       /* n_obs*2 pixel measurements (uv_in_image) */
  double huber_delta;         /* > 0: RobustKernel::Huber(delta); <= 0: no kernel.  A positive
                               * delta must be a normal float (1.2e-38 .. 3.4e38): the kernels
                               * compare residual norms with it in float */
} sgba_problem_desc;

/* OptParams fields used on this path (crates/sophus_opt/src/nlls/optimizer_types.rs:161-240).
 * Tolerances <= 0 disable the test, as 0.0 does in the reference. */
typedef struct {
  int32_t num_iterations;
  double initial_lm_damping;
  double function_tolerance;
  double gradient_tolerance;
  double parameter_tolerance;
  int64_t max_consecutive_rejects;
  int32_t skip_final_hessian;
} sgba_opt_params;

/* TerminationReason (crates/sophus_opt/src/nlls/optimizer_types.rs:93-122). */
typedef enum {
  SGBA_TERM_NONE = 0,
  SGBA_TERM_FUNCTION_TOLERANCE = 1,
  SGBA_TERM_GRADIENT_TOLERANCE = 2,
  SGBA_TERM_PARAMETER_TOLERANCE = 3,
  SGBA_TERM_MAX_ITERATIONS = 4,
  SGBA_TERM_MAX_CONSECUTIVE_REJECTS = 5,
} sgba_termination;

/* One record per Optimizer::step, mirroring StepInfo
 * (crates/sophus_opt/src/nlls/optimizer_types.rs:67-83) plus step diagnostics. */
typedef struct {
  double merit;        /* merit after the step */
  double new_merit;    /* cost at the trial point (NaN when no trial point was formed) */
  double lm_damping;   /* LM damping after the step */
  double gain_ratio;   /* NaN when not computed */
  double max_step;     /* max |delta| (NaN when no step) */
  double max_grad;     /* max |neg_gradient| at the linearisation point */
  int32_t accepted;
  int32_t termination; /* sgba_termination */
} sgba_iter_record;

typedef struct sgba_problem sgba_problem;

/* Version of this ABI (SGBA_ABI_VERSION). */
int32_t sgba_abi_version(void);

/* Copies the last error message of this thread into buf (NUL-terminated). */
size_t sgba_last_error(char *buf, size_t cap);

/* Validates and uploads a problem: sorts the cost terms as CostFn::sort does
 * (crates/sophus_opt/src/nlls/cost/cost_fn.rs:354-393), assigns free/marg
 * block indices (crates/sophus_opt/src/variables/var_families.rs:60-113) and
 * builds the Hessian and reduced-camera-system sparsity
 * (crates/sophus_opt/src/nlls/cost/cost_fn.rs:435-518,
 *  crates/sophus_opt/src/nlls/damped_hessian.rs:261-325).  device < 0 keeps
 * the current CUDA device. */
int sgba_problem_create(const sgba_problem_desc *desc, int32_t device, sgba_problem **out);

/* Options of sgba_problem_create_ex.
 *
 * camera_model selects the camera of every observation:
 *   SGBA_CAMERA_PINHOLE  params fx fy cx cy (PinholeCameraF64,
 *                        crates/sophus_sensor/src/camera_enum/perspective_camera.rs)
 *   SGBA_CAMERA_EUCM     the enhanced unified camera model, params fx fy cx cy
 *                        alpha beta (EnhancedUnifiedCameraF64,
 *                        crates/sophus_sensor/src/distortions/enhanced_unified.rs:55-215;
 *                        the camera of the reference's BA example problem,
 *                        crates/sophus_opt/src/example_problems/ba_problem.rs:69-110):
 *                        desc->intrinsics holds fx fy cx cy, eucm_alpha_beta
 *                        alpha beta.  For the pinhole eucm_alpha_beta is zero.
 * intrinsics_free = 1 makes the camera family Free (the reference's
 * VarKind::Free for the "cams" family: kinds (F, F, M), J_cam =
 * -dx_distort_params, pinhole_reprojection.rs:85): the camera's params (4 or
 * 6) are optimised with the poses, nu I per reduced term on their block, as
 * one more 6-row block of the reduced system (the pinhole's 4 rows padded).
 * The block comes first in the exported patterns and in
 * sgba_debug_last_system (the reference's family order).  Loop-shaped problems
 * (the banded solver) and PCG with free intrinsics are rejected with
 * SGBA_ERR_UNSUPPORTED. */
enum { SGBA_CAMERA_PINHOLE = 0, SGBA_CAMERA_EUCM = 1 };
typedef struct {
  int32_t intrinsics_free;     /* 0 Conditioned (default), 1 Free */
  int32_t camera_model;        /* SGBA_CAMERA_PINHOLE or SGBA_CAMERA_EUCM */
  double eucm_alpha_beta[2];   /* EUCM alpha beta (finite); zero for the pinhole */
  int32_t reserved[2];         /* zero */
} sgba_problem_options;
/* sgba_problem_create with options (NULL: the defaults). */
int sgba_problem_create_ex(const sgba_problem_desc *desc, const sgba_problem_options *options, int32_t device,
                           sgba_problem **out);

/* Pose-graph edges: a cost function of PoseGraph3CostTerm terms
 * (crates/sophus_opt/src/nlls/functor_library/costs/pose_graph3.rs) beside
 * the reprojection cost.  Edge k joins poses edge_pose[2k] = m and
 * edge_pose[2k + 1] = n (m != n) with the measured pose_m_from_pose_n
 * edge_m_from_n + 7k (qw qx qy qz tx ty tz); residual log(T_m^-1 T_n M^-1),
 * cost g^T g.  Edges with equal (m, n) form one reduced term.  A term between
 * two free poses adds their block to the reduced camera system; the edges
 * fix the scale (no gauge projection).  Not with free camera params. */
typedef struct {
  int32_t n_edge;
  const int32_t *edge_pose;      /* n_edge x 2 */
  const double *edge_m_from_n;   /* n_edge x 7 */
} sgba_pose_graph;
/* sgba_problem_create_ex with pose-graph edges (graph NULL or n_edge 0:
 * none).  Problems with edges run on their own streams in
 * sgba_batch_optimize. */
int sgba_problem_create_graph(const sgba_problem_desc *desc, const sgba_problem_options *options,
                              const sgba_pose_graph *graph, int32_t device, sgba_problem **out);
int sgba_problem_destroy(sgba_problem *p);

/* Optimizer::new: validates the solver configuration
 * (crates/sophus_opt/src/nlls/optimizer.rs:649-717), evaluates the initial
 * merit and resets damping / reject counters. */
int sgba_optimizer_init(sgba_problem *p, const sgba_opt_params *params);

/* Optimizer::step: one LM iteration; fills *record. */
int sgba_optimizer_step(sgba_problem *p, sgba_iter_record *record);

/* optimize_nlls: init, step until a termination reason, then build_solution.
 * Up to cap records are written; *n_records receives the number of steps. */
int sgba_optimize(sgba_problem *p, const sgba_opt_params *params, sgba_iter_record *records,
                  int32_t cap, int32_t *n_records, int32_t *termination);

/* Batched optimize_nlls over independent problems (the local windows of a
 * local bundle adjustment, 5-40 cameras each; in the reference one
 * optimize_nlls call per window, crates/sophus_opt/src/nlls.rs:73-83):
 * every window is an sgba_problem created as usual.  Windows on the FP32
 * linearization with the dense reduced-system solver (pinhole camera, fixed
 * intrinsics, no PCG) run batched: each kernel of an LM iteration is launched
 * once for all of them (block b of a launch runs block b - off[w] of window
 * w's own grid), one CUDA graph per LM iteration and window group; the other
 * windows run on their own streams alongside.  Per window the result is
 * exactly what sgba_optimize would return for it.  A batched window's
 * results[w].ms is the device time of the whole batched run.
 * records: NULL, or n * cap records (window w at records + w * cap);
 * results: n entries.  Returns SGBA_OK when the call itself is well formed;
 * per-window failures are reported in results[w].status.
 * Concurrent calls on one device are serialised. */
typedef struct {
  int32_t status;       /* sgba_status of this window */
  int32_t termination;  /* sgba_termination */
  int32_t n_records;    /* steps taken */
  float ms;             /* device time of the window (first iteration to final linearisation) */
  double final_cost;    /* merit after the last step */
} sgba_window_result;
int sgba_batch_optimize(sgba_problem *const *problems, int32_t n, const sgba_opt_params *params,
                        sgba_iter_record *records, int32_t cap, sgba_window_result *results);

/* What the last sgba_batch_optimize call of the process did on its batched
 * path (no counterpart in the reference).  The schedule -- window groups run
 * on separate streams, and whether windows are ordered by decreasing work --
 * never changes a window's results; an online autotuner times one LM
 * iteration per candidate on the first calls for a shape (window and
 * observation counts rounded to powers of two) and keeps the fastest. */
typedef struct {
  int32_t batched_windows;  /* windows run by the batched launches */
  int32_t schedule;         /* candidate used for the last iterations */
  int32_t groups;           /* its window groups (one stream and one graph each) */
  int32_t order;            /* 1: windows ordered by decreasing work, 0: as given */
  int32_t tuned;            /* 1: the autotuner has settled on a candidate for this shape */
  int32_t pad;
  int64_t kernel_launches;  /* kernels the batched path launched in the call */
  float ms;                 /* device time of the batched path (init to final linearisation) */
  float schedule_ms[4];     /* mean time of one LM iteration per candidate (0: not measured) */
} sgba_batch_stats;
int sgba_batch_last_stats(sgba_batch_stats *out);

/* Current variables (OptimizationSolution.variables). NULL skips a family. */
int sgba_get_variables(sgba_problem *p, double *poses, double *points);
/* Current camera params (changed by the optimisation when free): fx fy cx cy,
 * then alpha beta for the EUCM camera (4 or 6 doubles). */
int sgba_get_intrinsics(sgba_problem *p, double *intrinsics);
/* Current merit (OptimizationSolution.final_cost after sgba_optimize). */
int sgba_get_cost(sgba_problem *p, double *cost);
/* Overwrite the variables of an existing problem (same structure). */
int sgba_set_variables(sgba_problem *p, const double *poses, const double *points);

/* Pose priors: a second cost function of Isometry3PriorCostTerm terms
 * (crates/sophus_opt/src/nlls/functor_library/costs/isometry3_prior.rs,
 * tested by crates/sophus_opt/src/example_problems/cam_calib.rs:249-342).
 * Prior k on pose[k] has the mean pose mean + 7k (qw qx qy qz tx ty tz) and
 * the 6x6 precision precision + 36k (row-major); residual log(T E^-1), cost
 * g^T W g, no robust kernel.  A prior on a constant pose adds only its cost.
 * Replaces any earlier set (n = 0 removes them); takes effect at the next
 * sgba_optimizer_init / sgba_optimize.  With priors the scale gauge is held by
 * them (no gauge projection).  Windows with priors are not batched by
 * sgba_batch_optimize (they run on their own streams).  Not with free camera
 * params (SGBA_ERR_UNSUPPORTED). */
int sgba_set_pose_priors(sgba_problem *p, int32_t n, const int32_t *pose, const double *mean,
                         const double *precision);

/* Equality constraints |t(pose[k])| = radius[k] (TranslationNormConstraint,
 * crates/sophus_opt/src/example_problems/ba_scale_constraint.rs:57-100), at
 * most 8, each on a Free pose, solved with the LM step by the range-space KKT
 * method of the Schur solver (crates/sophus_solver/src/ldlt/schur_ldlt.rs:
 * 674-772): Y = S^-1 G^T, M = G Y, dlam = M^-1 (G S^-1 r + c), dx = S^-1 r - Y
 * dlam; the multipliers start at zero at sgba_optimizer_init and move by -dlam
 * with every accepted step (EqSystem::update_lambdas).  Only for reduced
 * systems on the one-CTA solver (at most 234 rows, not loop-shaped), exact
 * factorization (SGBA_ERR_UNSUPPORTED otherwise).  Replaces any earlier set
 * (n = 0 removes them); the scale gauge is then held by the constraints. */
int sgba_set_eq_constraints(sgba_problem *p, int32_t n, const int32_t *pose, const double *radius);

/* Sizes of the problem as laid out on the device. */
typedef struct {
  int32_t n_free_poses;     /* free pose blocks (6 dof) */
  int32_t n_marg_points;    /* marginalized point blocks (3 dof) */
  int64_t n_terms;          /* reduced cost terms (distinct (point, pose) pairs) */
  int64_t n_h_blocks;       /* lower blocks of H: pose diag + point diag + point x pose */
  int64_t n_s_blocks;       /* lower 6x6 blocks of the reduced camera system S */
  int64_t n_schur_pairs;    /* observation pairs summed into S (sum over points of L(L+1)/2) */
  int32_t solver;           /* reduced-system solver: SGBA_SOLVER_* */
  int32_t band_width;       /* banded solver: band width in scalars (row r holds columns r-w+1..r) */
  int32_t border_rows;      /* banded solver: dense border rows at the end (loop closures) */
  int32_t float_float_lin;  /* 1: Jacobians, products and Z in float-float (loop-shaped problems) */
  int32_t intrinsics_rows;  /* 6 when the intrinsics are free (their block in S), else 0 */
} sgba_layout;
/* Reduced camera system solvers (chosen at sgba_problem_create from the size
 * and the block pattern of S). */
enum {
  SGBA_SOLVER_DENSE_CLUSTER = 0, /* dense S in one thread-block cluster's shared memory */
  SGBA_SOLVER_BAND = 1,          /* band + dense border, float-float (sequential / loop problems) */
  SGBA_SOLVER_DENSE_PANELS = 2,  /* dense S, panel launches (large dense systems) */
  SGBA_SOLVER_DENSE_SMALL = 3    /* dense S of at most 144 rows: one CTA, float-float (local windows) */
};
int sgba_get_layout(sgba_problem *p, sgba_layout *out);

/* Block sparsity of H (lower: row block, col block in the global block order
 * free poses then marginalized points) and of S (free pose blocks).  Arrays
 * of length n_h_blocks / n_s_blocks (see sgba_get_layout); NULL skips one. */
int sgba_export_pattern(sgba_problem *p, int32_t *h_rows, int32_t *h_cols, int32_t *s_rows,
                        int32_t *s_cols);

/* Linear system of the most recent step: S (dense n x n, row-major, lower
 * triangle valid, n = intrinsics_rows + 6nf), reduced rhs (n) and the step
 * delta (n + 3nm); with free intrinsics their (padded) block comes first.
 * NULL skips an output.  Used to compare each LM step with an FP64 LDLT. */
int sgba_debug_last_system(sgba_problem *p, double *s_dense, double *rhs, double *delta);

/* Per-term Jacobians at the current variables, evaluated by the same device
 * code as the linearization: J_pose (2x6 row-major per term, left perturbation
 * exp(delta) * world_from_camera, delta = [omega; nu]) and J_point (2x3) of the
 * residual uv - proj(camera_from_world * point) of
 * PinholeCameraReprojectionCostTerm::eval
 * (crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:60-95),
 * which the reference evaluates with DualScalar forward mode.  One term per
 * (cam[i], pt[i]); precision 0 = FP32 (the linearization of well-conditioned
 * problems), 1 = float-float (loop-shaped problems and point blocks rebuilt in
 * float-float).  j_pose: n*12 doubles, j_point: n*6.  Synchronous. */
int sgba_debug_jacobians(sgba_problem *p, int64_t n, const int32_t *cam, const int32_t *pt, int32_t precision,
                         double *j_pose, double *j_point);

/* ---- covariance and precision queries of the solution ---------------------
 * Replaces OptimizationSolution::covariance_block / precision_block
 * (crates/sophus_opt/src/nlls/optimizer_types.rs:277-370) over the final
 * Hessian that Optimizer::build_solution evaluates with zero damping
 * (crates/sophus_opt/src/nlls/optimizer.rs:609-646), answered through the
 * Schur factor as SchurFactor::inverse_block does
 * (crates/sophus_solver/src/ldlt/schur_ldlt.rs:815-957):
 *   pose x pose    S^-1 block
 *   pose x point   -(S^-1 H_fm H_mm^-1) block (and its transpose)
 *   point x point  H_mm^-1 delta_ij + H_mm[i]^-1 H_mf_i S^-1 H_mf_j^T H_mm[j]^-1
 * with S^-1 the min-norm pseudo-inverse when the LDL^T of S has zero pivots
 * (min_norm_ldlt.rs:55-140).  All in f64 on the device.
 *
 * sgba_covariance_prepare evaluates H at the current variables (after
 * sgba_optimize: the solution), forms S, factors and inverts it; the queries
 * answer from that snapshot until the next prepare or release (like the
 * reference's solution object, later changes of the variables do not reach
 * it).  With Free camera params their block comes first (4 or 6 rows, the
 * reference's family order) and couples to every pose and point.  Problems
 * with equality constraints, and more than 4096 free poses, are
 * SGBA_ERR_UNSUPPORTED; an H_mm block with a zero
 * determinant or an S the factor rejects (a non-finite pivot, or an
 * indefinite block in the Bunch-Kaufman case) is SGBA_ERR_FACTORIZATION.
 * Memory: 2 (6 nf)^2 doubles for S and its inverse, 66 doubles per reduced
 * term. */
typedef struct {
  int32_t n;          /* rows of S (6 per free pose) */
  int32_t rank;       /* positive pivots of its LDL^T (n: S^-1; fewer: the min-norm pseudo-inverse) */
  int32_t kernel_launches;
  int32_t pad;
  double ms_assemble; /* device time: H blocks and S */
  double ms_factor;   /* LDL^T */
  double ms_inverse;  /* S^-1 or S+ */
} sgba_cov_info;
int sgba_covariance_prepare(sgba_problem *p, sgba_cov_info *info);
int sgba_covariance_release(sgba_problem *p);

/* Variable kinds of a query: the reference's variable families. */
enum {
  SGBA_VAR_INTRINSICS = 0, /* the camera params (index 0); a block only when they are Free */
  SGBA_VAR_POSE = 1,       /* index: pose (camera) index */
  SGBA_VAR_POINT = 2       /* index: point index */
};
typedef struct {
  int32_t row_kind;  /* SGBA_VAR_* */
  int32_t row_index;
  int32_t col_kind;
  int32_t col_index;
} sgba_cov_query;
enum {
  SGBA_QUERY_COVARIANCE = 0, /* covariance_block */
  SGBA_QUERY_PRECISION = 1   /* precision_block: the block of the undamped H */
};
/* n block queries in one launch.  out: 36 doubles per query (rows x cols,
 * row-major, rows 4 or 6 for the camera params, 6 for a pose and 3 for a
 * point); dims: 2 per query
 * (rows, cols), (0, 0) where the reference returns None (a constant pose or
 * point, Conditioned camera params, an index out of range).  Requires sgba_covariance_prepare (else
 * SGBA_ERR_STATE); an unknown kind or mode is SGBA_ERR_INVALID_ARGUMENT.
 * Synchronous. */
int sgba_covariance_blocks(sgba_problem *p, int32_t mode, int32_t n, const sgba_cov_query *queries, double *out,
                           int32_t *dims);

/* Opaque optimizer state (variables, damping, reject count, step count) for
 * resume: *size receives the byte size when buf is NULL. */
int sgba_state_save(sgba_problem *p, void *buf, size_t *size);
int sgba_state_load(sgba_problem *p, const void *buf, size_t size);

/* Per-kernel launch count and device time of the last sgba_optimize call
 * (instrumentation for benchmarks; times are CUDA-event based). */
typedef struct {
  int64_t kernel_launches;   /* launches of this library's kernels */
  double ms_total;           /* device time of the whole optimize call */
  double ms_linearize;       /* landmark + camera passes (per call, summed) */
  double ms_schur;           /* reduced camera system assembly */
  double ms_factor;          /* factorization + solves + refinement */
  double ms_update;          /* back-substitution, gauge projection, update */
  double ms_cost;            /* trial cost + decision */
} sgba_profile;
int sgba_get_profile(sgba_problem *p, sgba_profile *out);
/* Enable per-phase event timing (adds events between phases; off by default). */
int sgba_set_profiling(sgba_problem *p, int32_t enabled);

/* ---- benchmark instrumentation (no counterpart in the reference) ---------
 * Require sgba_optimizer_init.  Times come from CUDA events on the problem's
 * stream.  With flush_l2 != 0 a 256 MiB buffer is written before every timed
 * unit so each starts with a cold L2. */
typedef enum {
  SGBA_KERNEL_ITERATION = 0,   /* one whole LM iteration (the graph) */
  SGBA_KERNEL_SCHUR = 1,       /* reduced camera system assembly (k_schur) */
  SGBA_KERNEL_LANDMARK = 2,    /* landmark pass: point blocks, Cholesky, Z */
  SGBA_KERNEL_CAMERA = 3,      /* camera pass: pose blocks and reduced rhs */
  SGBA_KERNEL_COST = 4,        /* trial cost (float-float) */
  SGBA_KERNEL_FACTOR = 5,      /* factorization + solves + refinement (several kernels) */
  SGBA_KERNEL_BACKSUB = 6,     /* back-substitution */
} sgba_kernel_id;

/* Runs `iters` LM iterations (each its own graph launch); *ms_sum is the sum
 * of their device times, *launches the number of kernel launches. */
int sgba_bench_iterations(sgba_problem *p, int32_t iters, int32_t flush_l2, double *ms_sum,
                          int64_t *launches);
/* Re-launches one kernel (or kernel group) `reps` times on the current data;
 * *ms_avg is the mean device time per launch. */
int sgba_bench_kernel(sgba_problem *p, int32_t kernel, int32_t reps, int32_t flush_l2, double *ms_avg);

/* ---- iterative solve of the reduced camera system ------------------------
 * The reference solves S dx_f = b only exactly (block LDL^T, selected through
 * the closed LinearSolverEnum, crates/sophus_solver/src/lib.rs:295-318; the
 * Schur factor crates/sophus_solver/src/ldlt/schur_ldlt.rs:536-812).  These
 * entry points add preconditioned conjugate gradients (FP64, Jacobi-scaled
 * system, one cooperative launch) in front of the exact factorization: when
 * PCG reaches |b - S x| <= tolerance |b| (scaled system) within
 * max_iterations, its x is the step and the factorization is skipped;
 * otherwise the factorization runs as usual (the fallback), in the same LM
 * iteration.  The preconditioner is block-Jacobi per free pose (mode 1), or
 * block-Jacobi corrected by a learned 6x6 block per pose (mode 2):
 * P_j = C_j^-T (I + L_j L_j^T) C_j^-1, C_j C_j^T the pose's scaled diagonal
 * block, L_j from a message-passing network over the camera covisibility
 * graph (3 layers, hidden width 64, BF16 weights, FP32 accumulation).
 * Default: mode 0, the exact factorization alone. */
typedef enum {
  SGBA_LINSOLVE_EXACT = 0,
  SGBA_LINSOLVE_PCG_BLOCK_JACOBI = 1,
  SGBA_LINSOLVE_PCG_LEARNED = 2,
} sgba_linsolve_mode;
typedef struct {
  int32_t mode;            /* sgba_linsolve_mode */
  int32_t max_iterations;  /* PCG iteration cap (e.g. 50) */
  double tolerance;        /* relative residual (e.g. 1e-8) */
} sgba_linear_solver;
typedef struct sgba_pcg_model sgba_pcg_model;
/* Selects the reduced-system solver of a problem (the iteration graph is
 * captured again).  model: required for mode 2, on the problem's device; it
 * must stay alive while the problem uses it. */
int sgba_set_linear_solver(sgba_problem *p, const sgba_linear_solver *cfg, const sgba_pcg_model *model);
/* PCG counters since sgba_optimizer_init. */
typedef struct {
  int64_t solves;                 /* PCG solves */
  int64_t fallbacks;              /* of which fell back to the exact factorization */
  int64_t iterations;             /* PCG iterations in total */
  int32_t last_iterations;
  int32_t last_status;            /* 0 converged, 1 iteration cap, 2 breakdown, 3 barrier wait gave up */
  double last_relative_residual;
} sgba_pcg_stats;
int sgba_get_pcg_stats(sgba_problem *p, sgba_pcg_stats *out);
/* The network's parameters (FP32 master copy; the kernels read a BF16 copy). */
int32_t sgba_pcg_num_params(void);
/* A model on `device` (< 0: current) with seeded initial weights: Glorot
 * uniform hidden layers, output head at L_j = 0.1 I. */
int sgba_pcg_model_create(int32_t device, uint64_t seed, sgba_pcg_model **out);
int sgba_pcg_model_destroy(sgba_pcg_model *m);
int sgba_pcg_model_set_params(sgba_pcg_model *m, const float *params, int32_t n);
int sgba_pcg_model_get_params(const sgba_pcg_model *m, float *params, int32_t n);

/* Training of the learned preconditioner on reduced systems with their exact
 * solutions (no counterpart in the reference).  Loss of one system:
 * e = x* - P b, loss = e^T S e / x*^T S x* (Jacobi-scaled system), minimised
 * by Adam over the FP32 master weights; forward and backward are this
 * library's kernels (the forward is the inference arithmetic). */
typedef struct sgba_pcg_trainset sgba_pcg_trainset;
typedef struct {
  int32_t epochs;
  int32_t batch;          /* systems per Adam step */
  double learning_rate;
  uint64_t seed;          /* order of the systems in each epoch */
} sgba_pcg_train_params;
int sgba_pcg_trainset_create(int32_t device, sgba_pcg_trainset **out);
int sgba_pcg_trainset_destroy(sgba_pcg_trainset *t);
int32_t sgba_pcg_trainset_size(const sgba_pcg_trainset *t);
/* Appends a system given on the host: the lower blocks (s_rows[k] >= s_cols[k],
 * n_blocks x 36 doubles, row-major) of a Jacobi-scaled SPD S, b and the
 * solution x of S x = b (6 nf each). */
int sgba_pcg_trainset_add(sgba_pcg_trainset *t, int32_t nf, int64_t n_blocks, const int32_t *s_rows,
                          const int32_t *s_cols, const double *blocks, const double *b, const double *x);
/* Appends the reduced system of the problem's latest LM step, scaled, with
 * its solution by the exact factorization. */
int sgba_pcg_collect(sgba_problem *p, sgba_pcg_trainset *t);
/* Loss of one system and (grad != NULL) its gradient w.r.t. the parameters. */
int sgba_pcg_loss_grad(sgba_pcg_model *m, sgba_pcg_trainset *t, int32_t index, double *loss, float *grad,
                       int32_t n_grad);
/* Adam over the set; epoch_loss (NULL or tp->epochs entries): mean loss of
 * each epoch, evaluated before each system's update. */
int sgba_pcg_train(sgba_pcg_model *m, sgba_pcg_trainset *t, const sgba_pcg_train_params *tp, double *epoch_loss);
/* PCG on a stored system: mode 1 block-Jacobi, 2 learned (model). */
int sgba_pcg_evaluate(const sgba_pcg_model *m, sgba_pcg_trainset *t, int32_t index, int32_t mode,
                      int32_t max_iterations, double tolerance, int32_t *iterations, double *relative_residual,
                      int32_t *status);

/* ---- allocation-free total cost (no counterpart in the reference) --------
 * calc_total_cost of the reprojection cost (the value sgba_get_cost reports,
 * float-float on the GPU) over observations that the caller already holds in
 * device memory, for callers that must not allocate while they run: code
 * inside a pre-sized memory pool or a real-time loop, where a cudaMalloc
 * would synchronize the device, fragment the pool or fail under a fixed
 * budget.  It allocates nothing (no cudaMalloc, no library allocator): its
 * scratch is one static device array of 599,808 bytes sized for at most 4096
 * cameras, and n_cam above that is rejected with SGBA_ERR_INVALID_ARGUMENT.
 *
 * poses (7 doubles per camera, world-from-camera as in sgba_problem_desc),
 * points (3 per point), obs_cam, obs_pt, obs_uv (2 per observation) and cost
 * (1 double, written) are device pointers on the current device; intrinsics
 * (fx, fy, cx, cy) is a host array; huber_delta <= 0 means no robust kernel
 * (a positive delta must be a normal float, as in sgba_problem_desc).  The
 * device arrays must be aligned to their element: obs_uv to 16 bytes (its
 * (u, v) pairs are loaded together), the double arrays to 8 and the index
 * arrays to 4; a misaligned pointer is rejected with SGBA_ERR_INVALID_ARGUMENT.
 * The call is asynchronous on `stream` (a cudaStream_t; NULL is the legacy
 * default stream).  Nothing needs to be zeroed by the caller.  An observation
 * index out of range makes *cost NaN.
 *
 * The first call on each device does the set-up with that device current
 * (the scratch address and the loading of the kernels): make it before any
 * stream capture begins.  Calls that overlap on one device (other streams,
 * other threads) share the scratch and race: order them on one stream or
 * with events. */
int sgba_total_cost_noalloc(int32_t n_cam, const double *poses, int32_t n_pt, const double *points,
                            int64_t n_obs, const int32_t *obs_cam, const int32_t *obs_pt,
                            const double *obs_uv, const double *intrinsics, double huber_delta,
                            double *cost, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* SGBA_H */
