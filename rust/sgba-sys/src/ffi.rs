//! Raw declarations of the C ABI in `include/sgba.h` (libsgba.so), one to one.
//!
//! Every function returns an `sgba_status` (0 = OK, negative = error class
//! mirroring `NllsError`, crates/sophus_opt/src/nlls/optimizer_types.rs:422-504);
//! `sgba_last_error` gives the calling thread's last message. A problem handle
//! is not thread-safe and owns one CUDA stream.
#![allow(non_camel_case_types)]

use core::ffi::{c_char, c_int, c_void};
use core::marker::{PhantomData, PhantomPinned};

pub const SGBA_ABI_VERSION: i32 = 2;

// sgba_status
pub const SGBA_OK: c_int = 0;
pub const SGBA_ERR_INVALID_ARGUMENT: c_int = -1;
pub const SGBA_ERR_INVALID_PARAMS: c_int = -2;
pub const SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG: c_int = -3;
pub const SGBA_ERR_UNSUPPORTED: c_int = -4;
pub const SGBA_ERR_CUDA: c_int = -5;
pub const SGBA_ERR_OUT_OF_MEMORY: c_int = -6;
pub const SGBA_ERR_STATE: c_int = -7;
pub const SGBA_ERR_DEVICE_TIMEOUT: c_int = -8;
pub const SGBA_ERR_FACTORIZATION: c_int = -9;

// sgba_termination (TerminationReason, crates/sophus_opt/src/nlls/optimizer_types.rs:93-122)
pub const SGBA_TERM_NONE: i32 = 0;
pub const SGBA_TERM_FUNCTION_TOLERANCE: i32 = 1;
pub const SGBA_TERM_GRADIENT_TOLERANCE: i32 = 2;
pub const SGBA_TERM_PARAMETER_TOLERANCE: i32 = 3;
pub const SGBA_TERM_MAX_ITERATIONS: i32 = 4;
pub const SGBA_TERM_MAX_CONSECUTIVE_REJECTS: i32 = 5;

// reduced camera system solvers (sgba_layout::solver)
pub const SGBA_SOLVER_DENSE_CLUSTER: i32 = 0;
pub const SGBA_SOLVER_BAND: i32 = 1;
pub const SGBA_SOLVER_DENSE_PANELS: i32 = 2;
pub const SGBA_SOLVER_DENSE_SMALL: i32 = 3;

// sgba_kernel_id (benchmark instrumentation)
pub const SGBA_KERNEL_ITERATION: i32 = 0;
pub const SGBA_KERNEL_SCHUR: i32 = 1;
pub const SGBA_KERNEL_LANDMARK: i32 = 2;
pub const SGBA_KERNEL_CAMERA: i32 = 3;
pub const SGBA_KERNEL_COST: i32 = 4;
pub const SGBA_KERNEL_FACTOR: i32 = 5;
pub const SGBA_KERNEL_BACKSUB: i32 = 6;

/// Opaque problem handle.
#[repr(C)]
pub struct sgba_problem {
    _private: [u8; 0],
    _marker: PhantomData<(*mut u8, PhantomPinned)>,
}

/// Problem description: host arrays owned by the caller, copied by
/// `sgba_problem_create`. Families "cams" (Conditioned pinhole intrinsics),
/// "poses" (Free Isometry3F64 with const ids), "points" (Marginalized
/// VecF64<3> with const ids) and the PinholeCameraReprojectionCostTerm terms.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct sgba_problem_desc {
    pub n_cam: i32,
    /// n_cam * 7: world_from_camera params (qw qx qy qz tx ty tz)
    pub poses: *const f64,
    /// n_cam flags (1 = constant id), or null
    pub pose_const: *const u8,
    pub n_pt: i32,
    /// n_pt * 3 world points
    pub points: *const f64,
    /// n_pt flags, or null
    pub point_const: *const u8,
    /// fx fy cx cy (PinholeCameraF64 params)
    pub intrinsics: [f64; 4],
    pub n_obs: i64,
    /// pose index per observation (entity_indices[1])
    pub obs_cam: *const i32,
    /// point index per observation (entity_indices[2])
    pub obs_pt: *const i32,
    /// n_obs * 2 pixel measurements (uv_in_image)
    pub obs_uv: *const f64,
    /// > 0: RobustKernel::Huber(delta); <= 0: no kernel
    pub huber_delta: f64,
}

/// OptParams fields used on this path; tolerances <= 0 disable a test.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct sgba_opt_params {
    pub num_iterations: i32,
    pub initial_lm_damping: f64,
    pub function_tolerance: f64,
    pub gradient_tolerance: f64,
    pub parameter_tolerance: f64,
    pub max_consecutive_rejects: i64,
    pub skip_final_hessian: i32,
}

/// One record per Optimizer::step (StepInfo plus step diagnostics).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_iter_record {
    pub merit: f64,
    pub new_merit: f64,
    pub lm_damping: f64,
    pub gain_ratio: f64,
    pub max_step: f64,
    pub max_grad: f64,
    pub accepted: i32,
    pub termination: i32,
}

/// Result of one window of `sgba_batch_optimize`.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_window_result {
    pub status: i32,
    pub termination: i32,
    pub n_records: i32,
    pub ms: f32,
    pub final_cost: f64,
}

/// Pose-graph edges of `sgba_problem_create_graph`.
#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct sgba_pose_graph {
    pub n_edge: i32,
    pub edge_pose: *const i32,
    pub edge_m_from_n: *const f64,
}

/// What the last batched optimisation did on its batched path.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_batch_stats {
    pub batched_windows: i32,
    pub schedule: i32,
    pub groups: i32,
    pub order: i32,
    pub tuned: i32,
    pub pad: i32,
    pub kernel_launches: i64,
    pub ms: f32,
    pub schedule_ms: [f32; 4],
}

/// Sizes of a problem as laid out on the device.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_layout {
    pub n_free_poses: i32,
    pub n_marg_points: i32,
    pub n_terms: i64,
    pub n_h_blocks: i64,
    pub n_s_blocks: i64,
    pub n_schur_pairs: i64,
    pub solver: i32,
    pub band_width: i32,
    pub border_rows: i32,
    pub float_float_lin: i32,
    pub intrinsics_rows: i32,
}

/// Result of `sgba_covariance_prepare`: the order of S, the positive pivots of
/// its LDL^T (fewer than n: the min-norm pseudo-inverse) and device times.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_cov_info {
    pub n: i32,
    pub rank: i32,
    pub kernel_launches: i32,
    pub pad: i32,
    pub ms_assemble: f64,
    pub ms_factor: f64,
    pub ms_inverse: f64,
}

pub const SGBA_VAR_INTRINSICS: i32 = 0;
pub const SGBA_VAR_POSE: i32 = 1;
pub const SGBA_VAR_POINT: i32 = 2;
pub const SGBA_QUERY_COVARIANCE: i32 = 0;
pub const SGBA_QUERY_PRECISION: i32 = 1;

/// One block query: (row kind, row index) x (col kind, col index).
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_cov_query {
    pub row_kind: i32,
    pub row_index: i32,
    pub col_kind: i32,
    pub col_index: i32,
}

pub const SGBA_CAMERA_PINHOLE: i32 = 0;
pub const SGBA_CAMERA_EUCM: i32 = 1;

/// Options of `sgba_problem_create_ex`: the camera model (pinhole, or EUCM
/// with its alpha beta) and whether its params are free.
#[repr(C)]
#[derive(Debug, Clone, Copy, Default)]
pub struct sgba_problem_options {
    pub intrinsics_free: i32,
    pub camera_model: i32,
    pub eucm_alpha_beta: [f64; 2],
    pub reserved: [i32; 2],
}

/// Launch count and device times of the last `sgba_optimize`.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct sgba_profile {
    pub kernel_launches: i64,
    pub ms_total: f64,
    pub ms_linearize: f64,
    pub ms_schur: f64,
    pub ms_factor: f64,
    pub ms_update: f64,
    pub ms_cost: f64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default)]
pub struct sgba_linear_solver {
    pub mode: i32,
    pub max_iterations: i32,
    pub tolerance: f64,
}

#[repr(C)]
#[derive(Debug, Clone, Copy, Default)]
pub struct sgba_pcg_stats {
    pub solves: i64,
    pub fallbacks: i64,
    pub iterations: i64,
    pub last_iterations: i32,
    pub last_status: i32,
    pub last_relative_residual: f64,
}

pub const SGBA_LINSOLVE_EXACT: i32 = 0;
pub const SGBA_LINSOLVE_PCG_BLOCK_JACOBI: i32 = 1;
pub const SGBA_LINSOLVE_PCG_LEARNED: i32 = 2;

#[repr(C)]
#[derive(Debug, Clone, Copy, Default)]
pub struct sgba_pcg_train_params {
    pub epochs: i32,
    pub batch: i32,
    pub learning_rate: f64,
    pub seed: u64,
}

/// Opaque training set of the learned block preconditioner.
#[repr(C)]
pub struct sgba_pcg_trainset {
    _private: [u8; 0],
}

/// Opaque parameters of the learned block preconditioner.
#[repr(C)]
pub struct sgba_pcg_model {
    _private: [u8; 0],
}

extern "C" {
    pub fn sgba_abi_version() -> i32;
    pub fn sgba_last_error(buf: *mut c_char, cap: usize) -> usize;
    pub fn sgba_problem_create(desc: *const sgba_problem_desc, device: i32, out: *mut *mut sgba_problem) -> c_int;
    pub fn sgba_problem_create_ex(
        desc: *const sgba_problem_desc,
        options: *const sgba_problem_options,
        device: i32,
        out: *mut *mut sgba_problem,
    ) -> c_int;
    pub fn sgba_problem_create_graph(
        desc: *const sgba_problem_desc,
        options: *const sgba_problem_options,
        graph: *const sgba_pose_graph,
        device: i32,
        out: *mut *mut sgba_problem,
    ) -> c_int;
    pub fn sgba_get_intrinsics(p: *mut sgba_problem, intrinsics: *mut f64) -> c_int;
    pub fn sgba_problem_destroy(p: *mut sgba_problem) -> c_int;
    pub fn sgba_optimizer_init(p: *mut sgba_problem, params: *const sgba_opt_params) -> c_int;
    pub fn sgba_optimizer_step(p: *mut sgba_problem, record: *mut sgba_iter_record) -> c_int;
    pub fn sgba_optimize(
        p: *mut sgba_problem,
        params: *const sgba_opt_params,
        records: *mut sgba_iter_record,
        cap: i32,
        n_records: *mut i32,
        termination: *mut i32,
    ) -> c_int;
    pub fn sgba_batch_optimize(
        problems: *const *mut sgba_problem,
        n: i32,
        params: *const sgba_opt_params,
        records: *mut sgba_iter_record,
        cap: i32,
        results: *mut sgba_window_result,
    ) -> c_int;
    pub fn sgba_batch_last_stats(out: *mut sgba_batch_stats) -> c_int;
    pub fn sgba_set_eq_constraints(p: *mut sgba_problem, n: i32, pose: *const i32, radius: *const f64) -> c_int;
    pub fn sgba_set_pose_priors(
        p: *mut sgba_problem,
        n: i32,
        pose: *const i32,
        mean: *const f64,
        precision: *const f64,
    ) -> c_int;
    pub fn sgba_get_variables(p: *mut sgba_problem, poses: *mut f64, points: *mut f64) -> c_int;
    pub fn sgba_get_cost(p: *mut sgba_problem, cost: *mut f64) -> c_int;
    pub fn sgba_set_variables(p: *mut sgba_problem, poses: *const f64, points: *const f64) -> c_int;
    pub fn sgba_get_layout(p: *mut sgba_problem, out: *mut sgba_layout) -> c_int;
    pub fn sgba_export_pattern(
        p: *mut sgba_problem,
        h_rows: *mut i32,
        h_cols: *mut i32,
        s_rows: *mut i32,
        s_cols: *mut i32,
    ) -> c_int;
    pub fn sgba_debug_last_system(p: *mut sgba_problem, s_dense: *mut f64, rhs: *mut f64, delta: *mut f64) -> c_int;
    pub fn sgba_debug_jacobians(
        p: *mut sgba_problem,
        n: i64,
        cam: *const i32,
        pt: *const i32,
        precision: i32,
        j_pose: *mut f64,
        j_point: *mut f64,
    ) -> c_int;
    pub fn sgba_covariance_prepare(p: *mut sgba_problem, info: *mut sgba_cov_info) -> c_int;
    pub fn sgba_covariance_release(p: *mut sgba_problem) -> c_int;
    pub fn sgba_covariance_blocks(
        p: *mut sgba_problem,
        mode: i32,
        n: i32,
        queries: *const sgba_cov_query,
        out: *mut f64,
        dims: *mut i32,
    ) -> c_int;
    pub fn sgba_state_save(p: *mut sgba_problem, buf: *mut c_void, size: *mut usize) -> c_int;
    pub fn sgba_state_load(p: *mut sgba_problem, buf: *const c_void, size: usize) -> c_int;
    pub fn sgba_get_profile(p: *mut sgba_problem, out: *mut sgba_profile) -> c_int;
    pub fn sgba_set_profiling(p: *mut sgba_problem, enabled: i32) -> c_int;
    pub fn sgba_bench_iterations(
        p: *mut sgba_problem,
        iters: i32,
        flush_l2: i32,
        ms_sum: *mut f64,
        launches: *mut i64,
    ) -> c_int;
    pub fn sgba_bench_kernel(p: *mut sgba_problem, kernel: i32, reps: i32, flush_l2: i32, ms_avg: *mut f64) -> c_int;
    pub fn sgba_set_linear_solver(
        p: *mut sgba_problem,
        cfg: *const sgba_linear_solver,
        model: *const sgba_pcg_model,
    ) -> c_int;
    pub fn sgba_get_pcg_stats(p: *mut sgba_problem, out: *mut sgba_pcg_stats) -> c_int;
    pub fn sgba_pcg_num_params() -> i32;
    pub fn sgba_pcg_model_create(device: i32, seed: u64, out: *mut *mut sgba_pcg_model) -> c_int;
    pub fn sgba_pcg_model_destroy(m: *mut sgba_pcg_model) -> c_int;
    pub fn sgba_pcg_model_set_params(m: *mut sgba_pcg_model, params: *const f32, n: i32) -> c_int;
    pub fn sgba_pcg_model_get_params(m: *const sgba_pcg_model, params: *mut f32, n: i32) -> c_int;
    pub fn sgba_pcg_trainset_create(device: i32, out: *mut *mut sgba_pcg_trainset) -> c_int;
    pub fn sgba_pcg_trainset_destroy(t: *mut sgba_pcg_trainset) -> c_int;
    pub fn sgba_pcg_trainset_size(t: *const sgba_pcg_trainset) -> i32;
    pub fn sgba_pcg_trainset_add(
        t: *mut sgba_pcg_trainset,
        nf: i32,
        n_blocks: i64,
        s_rows: *const i32,
        s_cols: *const i32,
        blocks: *const f64,
        b: *const f64,
        x: *const f64,
    ) -> c_int;
    pub fn sgba_pcg_collect(p: *mut sgba_problem, t: *mut sgba_pcg_trainset) -> c_int;
    pub fn sgba_pcg_loss_grad(
        m: *mut sgba_pcg_model,
        t: *mut sgba_pcg_trainset,
        index: i32,
        loss: *mut f64,
        grad: *mut f32,
        n_grad: i32,
    ) -> c_int;
    pub fn sgba_pcg_train(
        m: *mut sgba_pcg_model,
        t: *mut sgba_pcg_trainset,
        tp: *const sgba_pcg_train_params,
        epoch_loss: *mut f64,
    ) -> c_int;
    pub fn sgba_pcg_evaluate(
        m: *const sgba_pcg_model,
        t: *mut sgba_pcg_trainset,
        index: i32,
        mode: i32,
        max_iterations: i32,
        tolerance: f64,
        iterations: *mut i32,
        relative_residual: *mut f64,
        status: *mut i32,
    ) -> c_int;
    pub fn sgba_total_cost_noalloc(
        n_cam: i32,
        poses: *const f64,
        n_pt: i32,
        points: *const f64,
        n_obs: i64,
        obs_cam: *const i32,
        obs_pt: *const i32,
        obs_uv: *const f64,
        intrinsics: *const f64,
        huber_delta: f64,
        cost: *mut f64,
        stream: *mut c_void,
    ) -> c_int;
}
