//! Rust binding of libsgba, the GB300 path of sophus_opt's
//! `optimize_nlls` for bundle adjustment (crates/sophus_opt/src/nlls.rs:73-83):
//! one CostFn of PinholeCameraReprojectionCostTerm (optionally Huber),
//! intrinsics Conditioned, poses Free with constant ids, points Marginalized,
//! `LinearSolverEnum::SchurBlockSparseLdlt`.
//!
//! [`ffi`] declares the C ABI of `include/sgba.h` one to one. The types here
//! wrap it: [`Problem`] owns a device-resident problem (destroyed on drop),
//! [`Problem::optimize`] is `optimize_nlls` (including `build_solution`'s final
//! linearisation), [`Problem::init`] / [`Problem::step`] are `Optimizer::new` /
//! `Optimizer::step`, and [`batch_optimize`] runs many independent problems
//! (local windows) concurrently on one GPU. Errors carry the status class
//! (mirroring `NllsError`, crates/sophus_opt/src/nlls/optimizer_types.rs:422-504)
//! and the library's message. With the `sophus` feature, [`sophus`] builds
//! the problem from sophus_opt's variable families and cost terms.

pub mod ffi;
#[cfg(feature = "sophus")]
pub mod sophus;

use core::ffi::{c_char, c_int, c_void};
use std::ffi::CStr;

/// Error class of a failed call.
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub enum ErrorKind {
    /// Bad pointer, size, index or non-finite input.
    InvalidArgument,
    /// A pose quaternion fails `| |q| - 1 | <= 1e-6` (from_params).
    InvalidParams,
    /// `NllsError::SchurMissingFreeOrMarg`.
    SchurMissingFreeOrMarg,
    /// A configuration outside this path.
    Unsupported,
    /// CUDA runtime failure.
    Cuda,
    /// Device or host memory exhausted.
    OutOfMemory,
    /// A call out of order (e.g. a step before init).
    State,
    /// A bounded device wait gave up.
    DeviceTimeout,
    /// Covariance: an H_mm block or S could not be factored.
    Factorization,
    /// A status this binding does not know.
    Unknown,
}

impl ErrorKind {
    fn from_status(status: c_int) -> Self {
        match status {
            ffi::SGBA_ERR_INVALID_ARGUMENT => Self::InvalidArgument,
            ffi::SGBA_ERR_INVALID_PARAMS => Self::InvalidParams,
            ffi::SGBA_ERR_SCHUR_MISSING_FREE_OR_MARG => Self::SchurMissingFreeOrMarg,
            ffi::SGBA_ERR_UNSUPPORTED => Self::Unsupported,
            ffi::SGBA_ERR_CUDA => Self::Cuda,
            ffi::SGBA_ERR_OUT_OF_MEMORY => Self::OutOfMemory,
            ffi::SGBA_ERR_STATE => Self::State,
            ffi::SGBA_ERR_DEVICE_TIMEOUT => Self::DeviceTimeout,
            ffi::SGBA_ERR_FACTORIZATION => Self::Factorization,
            _ => Self::Unknown,
        }
    }
}

/// A failed call: its status, class and message.
#[derive(Debug, Clone)]
pub struct Error {
    pub kind: ErrorKind,
    pub status: i32,
    pub message: String,
}

impl core::fmt::Display for Error {
    fn fmt(&self, f: &mut core::fmt::Formatter<'_>) -> core::fmt::Result {
        write!(f, "sgba status {} ({:?}): {}", self.status, self.kind, self.message)
    }
}

impl std::error::Error for Error {}

impl Error {
    fn from_status(status: c_int) -> Self {
        Self { kind: ErrorKind::from_status(status), status, message: last_error() }
    }

    fn invalid_argument(message: &str) -> Self {
        Self {
            kind: ErrorKind::InvalidArgument,
            status: ffi::SGBA_ERR_INVALID_ARGUMENT,
            message: message.to_string(),
        }
    }
}

/// The calling thread's last error message.
pub fn last_error() -> String {
    let mut buf = [0 as c_char; 1024];
    // SAFETY: the library writes at most `cap` bytes including the NUL.
    unsafe {
        ffi::sgba_last_error(buf.as_mut_ptr(), buf.len());
        CStr::from_ptr(buf.as_ptr()).to_string_lossy().into_owned()
    }
}

fn check(status: c_int) -> Result<(), Error> {
    if status == ffi::SGBA_OK {
        Ok(())
    } else {
        Err(Error::from_status(status))
    }
}

fn to_i32(n: usize, what: &str) -> Result<i32, Error> {
    i32::try_from(n).map_err(|_| Error::invalid_argument(what))
}

/// The OptParams fields used on this path, with the reference's defaults
/// (crates/sophus_opt/src/nlls/optimizer_types.rs:225-240). Tolerances <= 0
/// disable a test.
#[derive(Debug, Clone, Copy)]
pub struct OptParams {
    pub num_iterations: i32,
    pub initial_lm_damping: f64,
    pub function_tolerance: f64,
    pub gradient_tolerance: f64,
    pub parameter_tolerance: f64,
    pub max_consecutive_rejects: i64,
    pub skip_final_hessian: bool,
}

impl Default for OptParams {
    fn default() -> Self {
        Self {
            num_iterations: 100,
            initial_lm_damping: 10.0,
            function_tolerance: 1e-10,
            gradient_tolerance: 1e-14,
            parameter_tolerance: 1e-12,
            max_consecutive_rejects: 20,
            skip_final_hessian: false,
        }
    }
}

impl OptParams {
    fn raw(&self) -> ffi::sgba_opt_params {
        ffi::sgba_opt_params {
            num_iterations: self.num_iterations,
            initial_lm_damping: self.initial_lm_damping,
            function_tolerance: self.function_tolerance,
            gradient_tolerance: self.gradient_tolerance,
            parameter_tolerance: self.parameter_tolerance,
            max_consecutive_rejects: self.max_consecutive_rejects,
            skip_final_hessian: i32::from(self.skip_final_hessian),
        }
    }
}

/// One record per LM step (StepInfo plus step diagnostics).
pub type IterRecord = ffi::sgba_iter_record;

/// Sizes of a problem as laid out on the device.
pub type Layout = ffi::sgba_layout;

/// TerminationReason (crates/sophus_opt/src/nlls/optimizer_types.rs:93-122).
#[derive(Debug, Clone, Copy, PartialEq, Eq)]
pub enum Termination {
    None,
    FunctionTolerance,
    GradientTolerance,
    ParameterTolerance,
    MaxIterations,
    MaxConsecutiveRejects,
}

impl Termination {
    fn from_raw(t: i32) -> Self {
        match t {
            ffi::SGBA_TERM_FUNCTION_TOLERANCE => Self::FunctionTolerance,
            ffi::SGBA_TERM_GRADIENT_TOLERANCE => Self::GradientTolerance,
            ffi::SGBA_TERM_PARAMETER_TOLERANCE => Self::ParameterTolerance,
            ffi::SGBA_TERM_MAX_ITERATIONS => Self::MaxIterations,
            ffi::SGBA_TERM_MAX_CONSECUTIVE_REJECTS => Self::MaxConsecutiveRejects,
            _ => Self::None,
        }
    }
}

/// A bundle adjustment problem in host memory; the library copies it.
#[derive(Debug, Clone, Copy)]
pub struct BaProblem<'a> {
    /// world_from_camera params per pose: qw qx qy qz tx ty tz (Isometry3F64 params).
    pub poses: &'a [[f64; 7]],
    /// 1 = constant id, per pose.
    pub pose_const: Option<&'a [u8]>,
    /// World points.
    pub points: &'a [[f64; 3]],
    /// 1 = constant id, per point.
    pub point_const: Option<&'a [u8]>,
    /// fx fy cx cy (PinholeCameraF64 params; Conditioned).
    pub intrinsics: [f64; 4],
    /// Pose index per observation (entity_indices[1]).
    pub obs_cam: &'a [i32],
    /// Point index per observation (entity_indices[2]).
    pub obs_pt: &'a [i32],
    /// Pixel measurement per observation (uv_in_image).
    pub obs_uv: &'a [[f64; 2]],
    /// RobustKernel::Huber(delta), or no kernel.
    pub huber_delta: Option<f64>,
}

/// Outcome of an optimisation: the records of its steps, why it stopped and
/// the final merit.
#[derive(Debug, Clone)]
pub struct Solution {
    pub records: Vec<IterRecord>,
    pub termination: Termination,
    pub final_cost: f64,
}

/// The camera of every observation (`sgba_problem_options::camera_model`):
/// the pinhole (params fx fy cx cy, `BaProblem::intrinsics`) or the enhanced
/// unified camera model (EnhancedUnifiedCameraF64, params fx fy cx cy from
/// `BaProblem::intrinsics`, then alpha beta here).
#[derive(Debug, Clone, Copy, PartialEq)]
pub enum Camera {
    Pinhole,
    Eucm { alpha: f64, beta: f64 },
}

/// A device-resident problem (an `sgba_problem` handle); destroyed on drop.
/// It may move to another thread but is not shared between threads.
pub struct Problem {
    raw: *mut ffi::sgba_problem,
    n_cam: usize,
    n_pt: usize,
    n_cam_params: usize,
}

// SAFETY: a handle is used by one thread at a time (no Sync); the library
// keeps no thread affinity for it.
unsafe impl Send for Problem {}

impl Problem {
    /// `sgba_problem_create`: validates and uploads; `device` < 0 keeps the
    /// current CUDA device.
    pub fn new(p: &BaProblem<'_>, device: i32) -> Result<Self, Error> {
        Self::new_with_camera(p, Camera::Pinhole, false, device)
    }

    /// `sgba_problem_create_ex`: the camera model, and whether its params
    /// are a Free family (kinds F, F, M) optimised with the poses.
    pub fn new_with_camera(p: &BaProblem<'_>, camera: Camera, intrinsics_free: bool, device: i32) -> Result<Self, Error> {
        Self::new_with_graph(p, camera, intrinsics_free, &[], &[], device)
    }

    /// `sgba_problem_create_graph`: `new_with_camera` plus PoseGraph3 edges
    /// (pose_graph3.rs): (m, n) pose pairs and the measured pose_m_from_pose_n
    /// of each.
    pub fn new_with_graph(
        p: &BaProblem<'_>,
        camera: Camera,
        intrinsics_free: bool,
        edges: &[[i32; 2]],
        edges_m_from_n: &[[f64; 7]],
        device: i32,
    ) -> Result<Self, Error> {
        let n_obs = p.obs_cam.len();
        if p.obs_pt.len() != n_obs || p.obs_uv.len() != n_obs {
            return Err(Error::invalid_argument("observation arrays differ in length"));
        }
        if p.pose_const.is_some_and(|c| c.len() != p.poses.len()) {
            return Err(Error::invalid_argument("pose_const length differs from the pose count"));
        }
        if p.point_const.is_some_and(|c| c.len() != p.points.len()) {
            return Err(Error::invalid_argument("point_const length differs from the point count"));
        }
        let desc = ffi::sgba_problem_desc {
            n_cam: to_i32(p.poses.len(), "too many poses")?,
            poses: p.poses.as_ptr().cast::<f64>(),
            pose_const: p.pose_const.map_or(core::ptr::null(), <[u8]>::as_ptr),
            n_pt: to_i32(p.points.len(), "too many points")?,
            points: p.points.as_ptr().cast::<f64>(),
            point_const: p.point_const.map_or(core::ptr::null(), <[u8]>::as_ptr),
            intrinsics: p.intrinsics,
            n_obs: i64::try_from(n_obs).map_err(|_| Error::invalid_argument("too many observations"))?,
            obs_cam: p.obs_cam.as_ptr(),
            obs_pt: p.obs_pt.as_ptr(),
            obs_uv: p.obs_uv.as_ptr().cast::<f64>(),
            huber_delta: p.huber_delta.unwrap_or(0.0),
        };
        let (camera_model, eucm_alpha_beta, n_cam_params) = match camera {
            Camera::Pinhole => (ffi::SGBA_CAMERA_PINHOLE, [0.0, 0.0], 4),
            Camera::Eucm { alpha, beta } => (ffi::SGBA_CAMERA_EUCM, [alpha, beta], 6),
        };
        let opts = ffi::sgba_problem_options {
            intrinsics_free: i32::from(intrinsics_free),
            camera_model,
            eucm_alpha_beta,
            reserved: [0; 2],
        };
        let graph = ffi::sgba_pose_graph {
            n_edge: to_i32(edges.len(), "too many edges")?,
            edge_pose: edges.as_ptr().cast::<i32>(),
            edge_m_from_n: edges_m_from_n.as_ptr().cast::<f64>(),
        };
        if edges.len() != edges_m_from_n.len() {
            return Err(Error::invalid_argument("edge pose pairs and measurements differ in length"));
        }
        let mut raw = core::ptr::null_mut();
        // SAFETY: every pointer in `desc` and `graph` covers the length it
        // states and outlives the call (the library copies the data); `opts`
        // is a complete options struct.
        check(unsafe { ffi::sgba_problem_create_graph(&desc, &opts, &graph, device, &mut raw) })?;
        Ok(Self { raw, n_cam: p.poses.len(), n_pt: p.points.len(), n_cam_params })
    }

    /// Isometry3 pose priors (isometry3_prior.rs): pose indices, means
    /// (qw qx qy qz tx ty tz) and 6x6 precisions (row-major); an empty set
    /// removes them.
    pub fn set_pose_priors(&mut self, pose: &[i32], mean: &[[f64; 7]], precision: &[[f64; 36]]) -> Result<(), Error> {
        if mean.len() != pose.len() || precision.len() != pose.len() {
            return Err(Error::invalid_argument("prior arrays differ in length"));
        }
        let n = to_i32(pose.len(), "too many priors")?;
        // SAFETY: the slices hold n indices, n * 7 and n * 36 doubles.
        check(unsafe {
            ffi::sgba_set_pose_priors(self.raw, n, pose.as_ptr(), mean.as_ptr().cast::<f64>(),
                                      precision.as_ptr().cast::<f64>())
        })
    }

    /// Equality constraints |t(pose[k])| = radius[k] (TranslationNormConstraint);
    /// an empty set removes them.
    pub fn set_eq_constraints(&mut self, pose: &[i32], radius: &[f64]) -> Result<(), Error> {
        if radius.len() != pose.len() {
            return Err(Error::invalid_argument("constraint arrays differ in length"));
        }
        let n = to_i32(pose.len(), "too many constraints")?;
        // SAFETY: the slices hold n indices and n doubles.
        check(unsafe { ffi::sgba_set_eq_constraints(self.raw, n, pose.as_ptr(), radius.as_ptr()) })
    }

    /// `build_solution`'s final Hessian at the current variables, S, its
    /// LDL^T and its inverse (the min-norm pseudo-inverse when S is
    /// rank-deficient), on the device, for `covariance_block` /
    /// `precision_block`.
    pub fn covariance_prepare(&mut self) -> Result<ffi::sgba_cov_info, Error> {
        let mut info = ffi::sgba_cov_info::default();
        // SAFETY: `self.raw` is a live handle; `info` is writable.
        check(unsafe { ffi::sgba_covariance_prepare(self.raw, &mut info) })?;
        Ok(info)
    }

    /// Block queries (`OptimizationSolution::covariance_block` with
    /// `mode` = SGBA_QUERY_COVARIANCE, `precision_block` with
    /// SGBA_QUERY_PRECISION): per query the (rows, cols) block row-major, or
    /// None where the reference returns None.
    pub fn covariance_blocks(
        &mut self,
        mode: i32,
        queries: &[ffi::sgba_cov_query],
    ) -> Result<Vec<Option<(usize, usize, Vec<f64>)>>, Error> {
        let n = to_i32(queries.len(), "too many queries")?;
        let mut out = vec![0.0f64; 36 * queries.len().max(1)];
        let mut dims = vec![0i32; 2 * queries.len().max(1)];
        // SAFETY: `queries` holds n queries, `out` 36 n doubles, `dims` 2 n ints.
        check(unsafe {
            ffi::sgba_covariance_blocks(self.raw, mode, n, queries.as_ptr(), out.as_mut_ptr(), dims.as_mut_ptr())
        })?;
        Ok((0..queries.len())
            .map(|k| {
                let (r, c) = (dims[2 * k], dims[2 * k + 1]);
                if r <= 0 {
                    None
                } else {
                    let (r, c) = (r as usize, c as usize);
                    Some((r, c, out[36 * k..36 * k + r * c].to_vec()))
                }
            })
            .collect())
    }

    /// `Optimizer::new`: validates the solver configuration, evaluates the
    /// initial merit, resets damping and counters.
    pub fn init(&mut self, params: &OptParams) -> Result<(), Error> {
        // SAFETY: `self.raw` is a live handle.
        check(unsafe { ffi::sgba_optimizer_init(self.raw, &params.raw()) })
    }

    /// `Optimizer::step`: one LM iteration.
    pub fn step(&mut self) -> Result<IterRecord, Error> {
        let mut rec = IterRecord::default();
        // SAFETY: `self.raw` is a live handle; `rec` is writable.
        check(unsafe { ffi::sgba_optimizer_step(self.raw, &mut rec) })?;
        Ok(rec)
    }

    /// `optimize_nlls`: init, steps until a termination reason, then the
    /// final linearisation of `build_solution`.
    pub fn optimize(&mut self, params: &OptParams) -> Result<Solution, Error> {
        let cap = params.num_iterations.max(1);
        let mut records = vec![IterRecord::default(); cap as usize];
        let (mut n, mut term) = (0i32, 0i32);
        // SAFETY: `records` holds `cap` records.
        check(unsafe { ffi::sgba_optimize(self.raw, &params.raw(), records.as_mut_ptr(), cap, &mut n, &mut term) })?;
        records.truncate(n.clamp(0, cap) as usize);
        Ok(Solution { records, termination: Termination::from_raw(term), final_cost: self.cost()? })
    }

    /// Current variables: world_from_camera params per pose and the points.
    pub fn variables(&self) -> Result<(Vec<[f64; 7]>, Vec<[f64; 3]>), Error> {
        let mut poses = vec![[0.0; 7]; self.n_cam];
        let mut points = vec![[0.0; 3]; self.n_pt];
        // SAFETY: the buffers hold n_cam * 7 and n_pt * 3 doubles.
        check(unsafe {
            ffi::sgba_get_variables(self.raw, poses.as_mut_ptr().cast::<f64>(), points.as_mut_ptr().cast::<f64>())
        })?;
        Ok((poses, points))
    }

    /// Overwrites the variables (same structure).
    pub fn set_variables(&mut self, poses: &[[f64; 7]], points: &[[f64; 3]]) -> Result<(), Error> {
        if poses.len() != self.n_cam || points.len() != self.n_pt {
            return Err(Error::invalid_argument("variable counts differ from the problem's"));
        }
        // SAFETY: the slices hold n_cam * 7 and n_pt * 3 doubles.
        check(unsafe { ffi::sgba_set_variables(self.raw, poses.as_ptr().cast::<f64>(), points.as_ptr().cast::<f64>()) })
    }

    /// Current merit.
    pub fn cost(&self) -> Result<f64, Error> {
        let mut c = 0.0;
        // SAFETY: `self.raw` is a live handle.
        check(unsafe { ffi::sgba_get_cost(self.raw, &mut c) })?;
        Ok(c)
    }

    /// Current camera params: fx fy cx cy, then alpha beta for the EUCM
    /// camera (moved by the optimisation when they are free).
    pub fn intrinsics(&self) -> Result<Vec<f64>, Error> {
        let mut k = vec![0.0; self.n_cam_params];
        // SAFETY: `k` holds the 4 or 6 params of this problem's camera model.
        check(unsafe { ffi::sgba_get_intrinsics(self.raw, k.as_mut_ptr()) })?;
        Ok(k)
    }

    /// Sizes and the solver chosen for the reduced camera system.
    pub fn layout(&self) -> Result<Layout, Error> {
        let mut l = Layout::default();
        // SAFETY: `self.raw` is a live handle.
        check(unsafe { ffi::sgba_get_layout(self.raw, &mut l) })?;
        Ok(l)
    }

    /// Opaque optimizer state (variables, damping, counters) for resume.
    pub fn state_save(&self) -> Result<Vec<u8>, Error> {
        let mut size = 0usize;
        // SAFETY: a null buffer asks for the size only.
        check(unsafe { ffi::sgba_state_save(self.raw, core::ptr::null_mut(), &mut size) })?;
        let mut buf = vec![0u8; size];
        // SAFETY: `buf` holds `size` bytes.
        check(unsafe { ffi::sgba_state_save(self.raw, buf.as_mut_ptr().cast::<c_void>(), &mut size) })?;
        Ok(buf)
    }

    /// Restores a state written by [`Problem::state_save`] of the same problem.
    pub fn state_load(&mut self, blob: &[u8]) -> Result<(), Error> {
        // SAFETY: `blob` holds `blob.len()` bytes.
        check(unsafe { ffi::sgba_state_load(self.raw, blob.as_ptr().cast::<c_void>(), blob.len()) })
    }
}

impl Drop for Problem {
    fn drop(&mut self) {
        // SAFETY: `self.raw` is live and dropped once.
        unsafe {
            ffi::sgba_problem_destroy(self.raw);
        }
    }
}

/// Many independent problems (local windows), each optimised as
/// [`Problem::optimize`] would alone, concurrently on their own CUDA streams.
/// The outer error is a malformed call; per-window failures are per entry.
pub fn batch_optimize(problems: &mut [Problem], params: &OptParams) -> Result<Vec<Result<Solution, Error>>, Error> {
    let n = to_i32(problems.len(), "too many problems")?;
    let cap = params.num_iterations.max(1);
    let handles: Vec<*mut ffi::sgba_problem> = problems.iter().map(|p| p.raw).collect();
    let mut records = vec![IterRecord::default(); problems.len() * cap as usize];
    let mut results = vec![ffi::sgba_window_result::default(); problems.len()];
    // SAFETY: `handles` are live; `records` holds n * cap records and `results` n entries.
    check(unsafe {
        ffi::sgba_batch_optimize(handles.as_ptr(), n, &params.raw(), records.as_mut_ptr(), cap, results.as_mut_ptr())
    })?;
    let cap = cap as usize;
    Ok(results
        .iter()
        .enumerate()
        .map(|(w, r)| {
            if r.status == ffi::SGBA_OK {
                let k = (r.n_records.max(0) as usize).min(cap);
                Ok(Solution {
                    records: records[w * cap..w * cap + k].to_vec(),
                    termination: Termination::from_raw(r.termination),
                    final_cost: r.final_cost,
                })
            } else {
                Err(Error {
                    kind: ErrorKind::from_status(r.status),
                    status: r.status,
                    message: format!("window {w} failed"),
                })
            }
        })
        .collect())
}

/// Version of the C ABI the library implements.
pub fn abi_version() -> i32 {
    // SAFETY: no arguments.
    unsafe { ffi::sgba_abi_version() }
}
