/*
 * sgba_oracle.h -- CPU FP64 restatement of sophus-rs's Schur-complement
 * Levenberg-Marquardt bundle-adjustment inner loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the correctness oracle for the
 * GB300 path: only the test suite, the smoke check and the CPU-baseline leg
 * of bench.py load it, and only as the checker / the timed CPU reference.
 * The product (libsgba) never links, loads or calls it.
 *
 * Every routine cites the reference function it restates (paths relative to
 * the sophus-rs workspace root).  The reference itself is Rust and cannot be
 * built in this environment (no cargo/rustc, crates not vendored), so this is
 * a restatement, not a wrapper.  Bit-level parity with the reference is
 * unpinned where it depends on third-party arithmetic (nalgebra's 3x3
 * inverse, faer's AMD ordering, rayon's summation order); the restated
 * reference tolerance tests pin it at the reference's own tolerances.
 */
#ifndef SGBA_ORACLE_H
#define SGBA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* OptParams fields used on the BA path
 * (crates/sophus_opt/src/nlls/optimizer_types.rs:161-240). */
typedef struct {
  int32_t num_iterations;
  double initial_lm_damping;
  double function_tolerance;
  double gradient_tolerance;
  double parameter_tolerance;
  int64_t max_consecutive_rejects;
  int32_t emulate_fp32; /* 1: per-term blocks, H and S assembled in float
                           (studies the GPU's FP32 assembly); 0: all f64 */
} ora_params;

/* One StepInfo-like record per Optimizer::step
 * (crates/sophus_opt/src/nlls/optimizer_types.rs:67-83). */
typedef struct {
  double merit;       /* merit after the step */
  double new_merit;   /* cost at the trial point (NaN if no trial) */
  double lm_damping;  /* damping after the step's update */
  double gain_ratio;
  double max_step;    /* max |delta| */
  double max_grad;    /* max |neg_grad| */
  int32_t accepted;
  int32_t termination; /* ORA_TERM_* */
} ora_record;

enum {
  ORA_TERM_NONE = 0,
  ORA_TERM_FUNCTION_TOL = 1,
  ORA_TERM_GRADIENT_TOL = 2,
  ORA_TERM_PARAMETER_TOL = 3,
  ORA_TERM_MAX_ITERATIONS = 4,
  ORA_TERM_MAX_REJECTS = 5,
};

/* ---- geometry / per-term math (unit-level checks) ---------------------- */
void ora_se3_exp(const double tangent[6], double out_params[7]);
void ora_se3_mul(const double a[7], const double b[7], double out[7]);
void ora_se3_inverse(const double a[7], double out[7]);
/* Residual, analytic Jacobians (row-major 2x6 pose, 2x3 point), Huber
 * weight and cost of one PinholeCameraReprojectionCostTerm. */
void ora_eval_term(const double pose[7], const double point[3],
                   const double intr[4], const double uv[2], double huber,
                   double r[2], double j_pose[12], double j_point[6],
                   double *weight, double *cost);
/* Same Jacobians via forward-mode dual numbers (DualScalar restatement). */
void ora_eval_term_dual(const double pose[7], const double point[3],
                        const double intr[4], const double uv[2],
                        double j_pose[12], double j_point[6]);

/* One Isometry3PriorCostTerm: residual g = log(T E^-1) (tangent rotation
 * first), J (6x6 row-major) its derivative under exp(x) * T at x = 0 by dual
 * numbers, and cost g^T W g (isometry3_prior.rs; evaluated_term.rs:286-327). */
void ora_eval_prior(const double pose[7], const double mean[7], const double precision[36],
                    double r[6], double j_pose[36], double *cost);
/* One PoseGraph3CostTerm: g = log(T_m^-1 T_n M^-1), J_n the derivative of
 * log(a exp(x) b) at x = 0 with a = T_m^-1, b = T_n M^-1 (by dual numbers), J_m
 * = -J_n (6x6 row-major each), cost g^T g (pose_graph3.rs). */
void ora_eval_edge(const double pose_m[7], const double pose_n[7], const double m_from_n[7],
                   double r[6], double j_m[36], double j_n[36], double *cost);
/* SE(3) log (affine_group_template.rs:362-370), tangent (rotation, translation). */
void ora_se3_log(const double params[7], double out_tangent[6]);

/* ---- linear algebra ----------------------------------------------------- */
/* Block LDLT (6x6 blocks when bs=6) of a dense SPD/PSD matrix, solve A x = b.
 * Returns 0 on success, -1 on a non-finite pivot. */
int ora_block_ldlt_solve(int n, int bs, const double *a_rowmajor,
                         const double *b, double *x);

/* Min-norm pseudo-inverse of a dense symmetric PSD matrix through its block
 * LDL^T (bs x bs blocks): E G^-1 diag(d_J)^-1 G^-1 E^T as above.  Returns the
 * rank (the positive pivots), or a negative error. */
int ora_min_norm_pinv(int n, int bs, const double *a_rowmajor, double *out);

/* ---- whole problem ------------------------------------------------------ */
typedef struct {
  int32_t n_cam;
  const double *poses;         /* n_cam*7, world_from_camera (qw qx qy qz tx ty tz) */
  const uint8_t *pose_const;   /* n_cam or NULL */
  int32_t n_pt;
  const double *points;        /* n_pt*3 */
  const uint8_t *point_const;  /* n_pt or NULL */
  double intrinsics[4];        /* fx fy cx cy */
  int64_t n_obs;
  const int32_t *obs_cam;
  const int32_t *obs_pt;
  const double *obs_uv;        /* n_obs*2 */
  double huber_delta;          /* <= 0: no robust kernel */
  int32_t intrinsics_free;     /* 1: the intrinsics are one Free variable (family kinds
                                  (F, F, M) instead of (C, F, M)); 0: Conditioned */
  int32_t camera_model;        /* ORA_CAMERA_PINHOLE (params fx fy cx cy) or
                                  ORA_CAMERA_EUCM (fx fy cx cy alpha beta) */
  double eucm_alpha_beta[2];   /* alpha, beta of the EUCM model */
  int32_t n_eq;                /* equality constraints |t(pose)| = radius
                                  (TranslationNormConstraint, ba_scale_constraint.rs:44-100);
                                  0: unconstrained */
  const int32_t *eq_pose;      /* n_eq pose indices (each a Free pose) */
  const double *eq_radius;     /* n_eq target translation norms */
  int32_t n_prior;             /* Isometry3PriorCostTerm terms (isometry3_prior.rs): a second
                                  cost function, ahead of the reprojection one in the cost
                                  list as in cam_calib.rs:318-325; 0: none */
  const int32_t *prior_pose;   /* n_prior pose indices */
  const double *prior_mean;    /* n_prior x 7 prior means E (qw qx qy qz tx ty tz) */
  const double *prior_precision; /* n_prior x 36 precision matrices W, row-major */
  int32_t n_edge;              /* PoseGraph3CostTerm terms (pose_graph3.rs): a cost function
                                  between the priors and the reprojection one; 0: none */
  const int32_t *edge_pose;    /* n_edge x 2 pose indices (m, n), m != n */
  const double *edge_mn;       /* n_edge x 7 measured pose_m_from_pose_n */
} ora_problem;

enum {
  ORA_CAMERA_PINHOLE = 0, /* PinholeCamera: affine distortion (affine.rs:50-108) */
  ORA_CAMERA_EUCM = 1,    /* EnhancedUnifiedCamera (enhanced_unified.rs:55-215) */
};

/* Total cost at the given variables (calc_total_cost). */
double ora_total_cost(const ora_problem *p, int n_threads);

/* Dense damped normal equations over active scalars (the 4 intrinsics when
 * they are free, then free poses, then marginalized points): H (n x n,
 * row-major) and neg_grad (n). Returns n, or the required n when the buffers
 * are NULL. */
int64_t ora_dense_system(const ora_problem *p, double nu, double *h,
                         double *neg_grad);

/* One Schur solve (forward pass, block LDLT of S, back-substitution) at the
 * given variables with damping nu.  delta has n active scalars (layout of
 * ora_dense_system).  Optionally returns S (ns x ns row-major) and rhs_bar,
 * ns = 6 nf, plus 6 when the intrinsics are free: their block comes first,
 * padded to 6 rows with an identity.  Returns 0, or -1 on failure. */
int ora_schur_step(const ora_problem *p, double nu, int n_threads,
                   int emulate_fp32, double *delta, double *s_out,
                   double *rhs_bar_out);

/* optimize_nlls on this path.  poses_out/points_out receive the final
 * variables.  With equality constraints (n_eq > 0) each step is the KKT step
 * of ora_schur_kkt_step from multipliers that start at zero, the gain ratio
 * and the parameter test run over [dx; dlam] against [neg_grad + G^T lambda;
 * -c], the merit stays the cost alone, and the gradient test is skipped
 * (optimizer_step.rs:365-430, optimizer.rs:527-535).  Returns 0 or a
 * negative error code. */
int ora_optimize(const ora_problem *p, const ora_params *params,
                 int n_threads, ora_record *records, int cap, int *n_records,
                 double *poses_out, double *points_out);

/* ora_optimize that also returns the final intrinsics (6 doubles: fx fy cx
 * cy, then alpha beta of the EUCM model, zero for a pinhole; they change
 * only when p->intrinsics_free). */
int ora_optimize_ex(const ora_problem *p, const ora_params *params,
                    int n_threads, ora_record *records, int cap, int *n_records,
                    double *poses_out, double *points_out, double *intrinsics_out);

/* Jacobian of one term's residual with respect to the pinhole intrinsics
 * (fx, fy, cx, cy), row-major 2x4 (pinhole_reprojection.rs:85:
 * -dx_distort_params of the projected point, affine.rs:77-108). */
void ora_eval_term_intrinsics(const double pose[7], const double point[3],
                              const double intr[4], double j_cam[8]);

/* One term for either camera model: residual, J_pose (2x6), J_point (2x3)
 * and J_cam (2 x n_params, n_params = 4 or 6), row-major; intr holds the
 * model's params (pinhole_reprojection.rs:60-95, ba_problem.rs:69-110). */
void ora_eval_term_ex(const double pose[7], const double point[3],
                      const double intr[6], int32_t camera_model, const double uv[2],
                      double r[2], double j_pose[12], double j_point[6],
                      double j_cam[12]);

/* Covariance block between two variables: a block of the inverse of the
 * undamped H at the given variables, through the Schur complement as
 * SchurFactor::inverse_block computes it (crates/sophus_solver/src/ldlt/schur_ldlt.rs:815-957):
 *   free x free  S^-1[row, col]
 *   free x marg  -(S^-1 H_fm H_mm^-1)[row, col]
 *   marg x marg  H_mm^-1 delta_ij + H_mm[i]^-1 H_mf_i S^-1 H_mf_j^T H_mm[j]^-1
 * Kinds: ORA_VAR_INTRINSICS (index ignored; only when they are free),
 * ORA_VAR_POSE (pose index), ORA_VAR_POINT (point index).  out receives the
 * rows x cols block row-major (4 or 6 intrinsics, 6 per pose, 3 per point).
 * When S is rank-deficient (a free gauge: no pose held), S^-1 above is the
 * min-norm pseudo-inverse E G^-1 diag(d_J)^-1 G^-1 E^T of its LDL^T factor
 * (min_norm_ldlt.rs:55-140, block_sparse_min_norm_ldlt.rs:98-160).
 * Returns 0; -1 for a variable without a block (constant or Conditioned, where
 * the reference returns None); -2 when S cannot be factored. */
enum {
  ORA_VAR_INTRINSICS = 0,
  ORA_VAR_POSE = 1,
  ORA_VAR_POINT = 2,
};
int ora_covariance_block(const ora_problem *p, int32_t row_kind, int32_t row_index,
                         int32_t col_kind, int32_t col_index, double *out,
                         int32_t *rows, int32_t *cols);

/* ---- equality constraints (Schur path, range-space KKT) ------------------ */
/* Residuals c_k = |t(T_k)| - r_k of the problem's TranslationNormConstraint
 * terms at the given poses (n_cam x 7), and their Jacobians under the left
 * perturbation exp(x) * T at x = 0, row-major n_eq x 6
 * (ba_scale_constraint.rs:64-100). */
void ora_eq_eval(const ora_problem *p, const double *poses, double *c, double *jac);

/* One damped step with the equality constraints, at the problem's variables
 * and the multipliers lambda (n_eq): the KKT system
 *   [H   G^T] [dx  ]   [neg_grad + G^T lambda]
 *   [G   0  ] [dlam] = [-c                   ]
 * solved as SchurFactor::solve does it (schur_ldlt.rs:756-812): points
 * eliminated, then u = S^-1 rhs_bar, dlam = (G S^-1 G^T)^-1 (G u + c),
 * dx_f = S^-1 (rhs_bar - G^T dlam), points back-substituted.  delta receives
 * n + n_eq entries: dx in the layout of ora_dense_system, then dlam.  The
 * multipliers then move as lambda <- lambda - dlam (EqSystem::update_lambdas).
 * Returns 0; -1 when S cannot be factored; -2 for a singular G S^-1 G^T
 * (SingularKktConstraint). */
int ora_schur_kkt_step(const ora_problem *p, double nu, const double *lambda, int n_threads,
                       double *delta);

#ifdef __cplusplus
}
#endif
#endif
