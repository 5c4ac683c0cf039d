//! Front over sophus_opt's types (feature `sophus`, sophus-rs 0.16): the
//! bundle-adjustment case of `optimize_nlls` (crates/sophus_opt/src/nlls.rs:73-83)
//! given as the variable families and the PinholeCameraReprojectionCostTerm
//! collection that would go into its `CostTerms`
//! (crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:28-95).
//!
//! The families must have the kinds of this path: intrinsics (PinholeCameraF64)
//! Conditioned with one member used by every term, poses (Isometry3F64) Free
//! (constant ids allowed), points (VecF64<3>) Marginalized (constant ids
//! allowed). Anything else is `ErrorKind::Unsupported`; the caller then runs
//! the reference's own `optimize_nlls`.

use sophus_autodiff::linalg::VecF64;
use sophus_autodiff::prelude::*;
use sophus_lie::prelude::*;
use sophus_lie::Isometry3F64;
use sophus_opt::nlls::costs::PinholeCameraReprojectionCostTerm;
use sophus_opt::variables::{IsVarFamily, VarFamilies, VarFamily, VarKind};
use sophus_sensor::PinholeCameraF64;

use crate::{BaProblem, Error, ErrorKind, OptParams, Problem, Solution};

/// Names of the three variable families, in `CostTerms::new` order.
#[derive(Debug, Clone, Copy)]
pub struct BaFamilies<'a> {
    pub cams: &'a str,
    pub poses: &'a str,
    pub points: &'a str,
}

/// Optimised variables (in the families' member order) and the run's records;
/// the device problem stays with them for `OptimizationSolution`'s
/// covariance and precision queries.
pub struct BaOutcome {
    pub world_from_cameras: Vec<Isometry3F64>,
    pub points: Vec<VecF64<3>>,
    pub solution: Solution,
    problem: Problem,
    families: [String; 3],
    cov_ready: bool,
}

impl BaOutcome {
    fn kind(&self, family: &str) -> Option<i32> {
        if family == self.families[0] {
            Some(crate::ffi::SGBA_VAR_INTRINSICS)
        } else if family == self.families[1] {
            Some(crate::ffi::SGBA_VAR_POSE)
        } else if family == self.families[2] {
            Some(crate::ffi::SGBA_VAR_POINT)
        } else {
            None
        }
    }

    fn query(
        &mut self,
        mode: i32,
        row_family: &str,
        row_var_idx: usize,
        col_family: &str,
        col_var_idx: usize,
    ) -> Result<Option<(usize, usize, Vec<f64>)>, Error> {
        let (Some(rk), Some(ck)) = (self.kind(row_family), self.kind(col_family)) else {
            return Ok(None);
        };
        if !self.cov_ready {
            self.problem.covariance_prepare()?;
            self.cov_ready = true;
        }
        let idx = |i: usize| i32::try_from(i).map_err(|_| Error::invalid_argument("variable index out of range"));
        let q = crate::ffi::sgba_cov_query { row_kind: rk, row_index: idx(row_var_idx)?, col_kind: ck, col_index: idx(col_var_idx)? };
        Ok(self.problem.covariance_blocks(mode, &[q])?.pop().flatten())
    }

    /// `OptimizationSolution::covariance_block` (optimizer_types.rs:319-370):
    /// (rows, cols, row-major values), or None for a constant variable or a
    /// Conditioned family.
    pub fn covariance_block(
        &mut self,
        row_family: &str,
        row_var_idx: usize,
        col_family: &str,
        col_var_idx: usize,
    ) -> Result<Option<(usize, usize, Vec<f64>)>, Error> {
        self.query(crate::ffi::SGBA_QUERY_COVARIANCE, row_family, row_var_idx, col_family, col_var_idx)
    }

    /// `OptimizationSolution::precision_block`: the block of the undamped H.
    pub fn precision_block(
        &mut self,
        row_family: &str,
        row_var_idx: usize,
        col_family: &str,
        col_var_idx: usize,
    ) -> Result<Option<(usize, usize, Vec<f64>)>, Error> {
        self.query(crate::ffi::SGBA_QUERY_PRECISION, row_family, row_var_idx, col_family, col_var_idx)
    }
}

fn unsupported(message: String) -> Error {
    Error { kind: ErrorKind::Unsupported, status: crate::ffi::SGBA_ERR_UNSUPPORTED, message }
}

fn kind_of<T: IsVarFamily + 'static>(variables: &VarFamilies, name: &str) -> Result<VarKind, Error> {
    variables
        .get::<T>(name)
        .map(|f| f.get_var_kind())
        .map_err(|e| unsupported(format!("family {name}: {e:?}")))
}

/// Optimises on the GPU (`device` < 0: the current CUDA device) and returns the
/// new poses and points; `huber_delta` is the delta of
/// `RobustKernel::Huber` when the cost function has one.
pub fn optimize_ba(
    variables: &VarFamilies,
    families: &BaFamilies<'_>,
    terms: &[PinholeCameraReprojectionCostTerm],
    huber_delta: Option<f64>,
    params: &OptParams,
    device: i32,
) -> Result<BaOutcome, Error> {
    if kind_of::<VarFamily<PinholeCameraF64>>(variables, families.cams)? != VarKind::Conditioned {
        return Err(unsupported("intrinsics must be Conditioned".into()));
    }
    if kind_of::<VarFamily<Isometry3F64>>(variables, families.poses)? != VarKind::Free {
        return Err(unsupported("poses must be Free".into()));
    }
    if kind_of::<VarFamily<VecF64<3>>>(variables, families.points)? != VarKind::Marginalized {
        return Err(unsupported("points must be Marginalized".into()));
    }
    let cams = variables.get_members::<PinholeCameraF64>(families.cams);
    let cam = terms.first().map_or(0, |t| t.entity_indices[0]);
    if terms.iter().any(|t| t.entity_indices[0] != cam) || cam >= cams.len().max(1) {
        return Err(unsupported("all terms must use one intrinsics member".into()));
    }
    let intr = cams.get(cam).map(|c| c.params().clone());
    let intrinsics = intr.map_or([0.0; 4], |p| [p[0], p[1], p[2], p[3]]);

    let poses_in = variables.get_members::<Isometry3F64>(families.poses);
    let points_in = variables.get_members::<VecF64<3>>(families.points);
    let poses: Vec<[f64; 7]> = poses_in
        .iter()
        .map(|t| {
            let p = t.params();
            [p[0], p[1], p[2], p[3], p[4], p[5], p[6]]
        })
        .collect();
    let points: Vec<[f64; 3]> = points_in.iter().map(|p| [p[0], p[1], p[2]]).collect();
    // constant ids have no block in their family's partition
    let pose_const: Vec<u8> =
        (0..poses.len()).map(|j| u8::from(variables.block_index(families.poses, j).is_none())).collect();
    let point_const: Vec<u8> =
        (0..points.len()).map(|i| u8::from(variables.block_index(families.points, i).is_none())).collect();

    let mut obs_cam = Vec::with_capacity(terms.len());
    let mut obs_pt = Vec::with_capacity(terms.len());
    let mut obs_uv = Vec::with_capacity(terms.len());
    for t in terms {
        let (j, i) = (t.entity_indices[1], t.entity_indices[2]);
        obs_cam.push(i32::try_from(j).map_err(|_| Error::invalid_argument("pose index out of range"))?);
        obs_pt.push(i32::try_from(i).map_err(|_| Error::invalid_argument("point index out of range"))?);
        obs_uv.push([t.uv_in_image[0], t.uv_in_image[1]]);
    }

    let mut problem = Problem::new(
        &BaProblem {
            poses: &poses,
            pose_const: Some(&pose_const),
            points: &points,
            point_const: Some(&point_const),
            intrinsics,
            obs_cam: &obs_cam,
            obs_pt: &obs_pt,
            obs_uv: &obs_uv,
            huber_delta,
        },
        device,
    )?;
    let solution = problem.optimize(params)?;
    let (poses_out, points_out) = problem.variables()?;
    Ok(BaOutcome {
        world_from_cameras: poses_out.iter().map(|p| Isometry3F64::from_params(VecF64::<7>::from_column_slice(p))).collect(),
        points: points_out.iter().map(|p| VecF64::<3>::new(p[0], p[1], p[2])).collect(),
        solution,
        problem,
        families: [families.cams.to_string(), families.poses.to_string(), families.points.to_string()],
        cov_ready: false,
    })
}
