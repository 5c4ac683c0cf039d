"""Python mirror of the sophus_opt API surface for the Schur-LM BA path.

Names, argument meaning and errors follow the reference crate so that a
caller of optimize_nlls / Optimizer on the bundle-adjustment path can switch
to the GB300 backend:

  optimize_nlls            crates/sophus_opt/src/nlls.rs:73-83
  Optimizer                crates/sophus_opt/src/nlls/optimizer.rs:71-120,345,609
  OptParams                crates/sophus_opt/src/nlls/optimizer_types.rs:161-240
  StepInfo / Termination   crates/sophus_opt/src/nlls/optimizer_types.rs:67-122
  VarKind / VarFamily      crates/sophus_opt/src/variables.rs:15-24, variables/var_family.rs
  VarBuilder               crates/sophus_opt/src/variables/var_builder.rs:16-50
  CostTerms / CostFn       crates/sophus_opt/src/nlls/cost/cost_term.rs:98, cost/cost_fn.rs:127-152
  HuberKernel              crates/sophus_opt/src/robust_kernel.rs
  PinholeCameraReprojectionCostTerm
                           crates/sophus_opt/src/nlls/functor_library/costs/pinhole_reprojection.rs:28-95
  EucmCameraReprojectionCostTerm
                           crates/sophus_opt/src/example_problems/ba_problem.rs:69-110
  PinholeCameraF64 / EnhancedUnifiedCameraF64
                           crates/sophus_sensor/src/camera_enum/perspective_camera.rs:53-71

Only the bundle-adjustment specialisation runs here (pinhole or EUCM
reprojection, intrinsics Conditioned or Free, poses Free, points
Marginalized, a Schur solver); other configurations raise NotOnGpuPath.
"""
import enum
from collections import OrderedDict
from dataclasses import dataclass, field
from typing import Any, List, Optional

import numpy as np

from . import native
from .synth import BAProblem


# ---------------------------------------------------------------- errors ----
class NllsError(Exception):
    """NllsError (crates/sophus_opt/src/nlls/optimizer_types.rs:422-504)."""


class SchurMissingFreeOrMarg(NllsError):
    pass


class SchurCostConnectsTwoMargFamilies(NllsError):
    pass


class SolverDoesNotSupportEqConstraints(NllsError):
    pass


class LinearSolverError(NllsError):
    pass


class NotOnGpuPath(NllsError):
    """The problem is outside the bundle-adjustment path this backend implements."""


# ------------------------------------------------------------- variables ----
class VarKind(enum.Enum):
    Free = "Free"
    Conditioned = "Conditioned"
    Marginalized = "Marginalized"


class Isometry3F64:
    """SE(3) as params [qw, qx, qy, qz, tx, ty, tz] (sophus_lie Isometry3F64)."""

    __slots__ = ("_p",)

    def __init__(self, params):
        p = np.asarray(params, dtype=np.float64).reshape(7).copy()
        n = np.linalg.norm(p[:4])
        if abs(n - 1.0) > 1e-6:  # are_params_valid (rotation3.rs:314-319)
            raise ValueError("Invalid parameters for Isometry3F64: %s" % p)
        if p[0] < 0.0:  # disambiguate (rotation3.rs:176-182)
            p[:4] = -p[:4]
        self._p = p

    @staticmethod
    def identity():
        return Isometry3F64([1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0])

    @staticmethod
    def from_rotation_and_translation(quat_wxyz, translation):
        return Isometry3F64(np.concatenate([np.asarray(quat_wxyz, float), np.asarray(translation, float)]))

    def params(self):
        return self._p.copy()

    def translation(self):
        return self._p[4:].copy()

    def __repr__(self):
        return "Isometry3F64(%s)" % np.array2string(self._p, precision=6)


class PinholeCameraF64:
    """Pinhole camera with params [fx, fy, cx, cy] (sophus_sensor PinholeCameraF64)."""

    def __init__(self, params, image_size=(640, 480)):
        self.params = np.asarray(params, dtype=np.float64).reshape(4).copy()
        self.image_size = tuple(image_size)

    @staticmethod
    def from_params_and_size(params, image_size):
        return PinholeCameraF64(params, image_size)


class EnhancedUnifiedCameraF64:
    """Enhanced unified camera with params [fx, fy, cx, cy, alpha, beta]
    (sophus_sensor EnhancedUnifiedCameraF64)."""

    def __init__(self, params, image_size=(640, 480)):
        self.params = np.asarray(params, dtype=np.float64).reshape(6).copy()
        self.image_size = tuple(image_size)

    @staticmethod
    def from_params_and_size(params, image_size):
        return EnhancedUnifiedCameraF64(params, image_size)


class VarFamily:
    """A family of variables of one type (var_family.rs)."""

    def __init__(self, kind, members, constant_ids=None):
        if not isinstance(kind, VarKind):
            raise TypeError("kind must be a VarKind")
        self.kind = kind
        self.members = members
        self.constant_ids = set(int(i) for i in (constant_ids or []))

    @staticmethod
    def new(kind, members):
        return VarFamily(kind, members)

    @staticmethod
    def new_with_const_ids(kind, members, constant_ids):
        return VarFamily(kind, members, list(constant_ids))

    def get_var_kind(self):
        return self.kind

    def __len__(self):
        return len(self.members)

    def dof(self):
        m = self.members
        if isinstance(m, np.ndarray):
            return 6 if m.shape[-1] == 7 else m.shape[-1]
        first = m[0] if len(m) else None
        if isinstance(first, Isometry3F64):
            return 6
        if isinstance(first, PinholeCameraF64):
            return 4
        if isinstance(first, EnhancedUnifiedCameraF64):
            return 6
        return int(np.asarray(first).size)

    def num_active(self):
        return len(self) - len(self.constant_ids)


class VarFamilies:
    """Families ordered by name, as the reference's BTreeMap is."""

    def __init__(self, families):
        self.collection = OrderedDict(sorted(families.items()))

    def get_members(self, name):
        return self.collection[name].members

    def num_free_scalars(self):
        return sum(f.num_active() * f.dof() for f in self.collection.values() if f.kind == VarKind.Free)

    def num_marg_scalars(self):
        return sum(f.num_active() * f.dof() for f in self.collection.values() if f.kind == VarKind.Marginalized)


class VarBuilder:
    def __init__(self):
        self._families = {}

    @staticmethod
    def new():
        return VarBuilder()

    def add_family(self, name, family):
        self._families[name] = family
        return self

    def build(self):
        return VarFamilies(self._families)


# ------------------------------------------------------------------ costs ----
@dataclass
class PinholeCameraReprojectionCostTerm:
    """uv_in_image, entity_indices = [intrinsics, pose, point]."""

    uv_in_image: Any
    entity_indices: Any


@dataclass
class EucmCameraReprojectionCostTerm:
    """uv_in_image, entity_indices = [intrinsics, pose, point] (EUCM camera)."""

    uv_in_image: Any
    entity_indices: Any


@dataclass
class Isometry3PriorCostTerm:
    """isometry_prior_mean (an Isometry3F64 or 7 params), isometry_prior_precision
    (6x6), entity_indices = [pose] (isometry3_prior.rs)."""

    isometry_prior_mean: Any
    isometry_prior_precision: Any
    entity_indices: Any


class PriorTerms:
    """Struct-of-arrays container of Isometry3PriorCostTerm terms."""

    def __init__(self, pose, mean, precision):
        self.pose = np.ascontiguousarray(pose, dtype=np.int32).reshape(-1)
        self.mean = np.ascontiguousarray(mean, dtype=np.float64).reshape(-1, 7)
        self.precision = np.ascontiguousarray(precision, dtype=np.float64).reshape(-1, 6, 6)
        if not (self.pose.shape[0] == self.mean.shape[0] == self.precision.shape[0]):
            raise ValueError("prior poses, means and precisions differ in length")

    def __len__(self):
        return self.pose.shape[0]


class PinholeReprojectionTerms:
    """Struct-of-arrays container of many PinholeCameraReprojectionCostTerm."""

    def __init__(self, uv_in_image, entity_indices):
        self.uv_in_image = np.ascontiguousarray(uv_in_image, dtype=np.float64).reshape(-1, 2)
        self.entity_indices = np.ascontiguousarray(entity_indices, dtype=np.int64).reshape(-1, 3)
        if self.uv_in_image.shape[0] != self.entity_indices.shape[0]:
            raise ValueError("uv_in_image and entity_indices differ in length")

    def __len__(self):
        return self.uv_in_image.shape[0]


class EucmReprojectionTerms(PinholeReprojectionTerms):
    """Struct-of-arrays container of many EucmCameraReprojectionCostTerm."""


class CostTerms:
    def __init__(self, family_names, terms):
        self.family_names = list(family_names)
        if isinstance(terms, (PinholeReprojectionTerms, PriorTerms)):
            self.terms = terms
        else:
            terms = list(terms)
            kinds = {type(t) for t in terms}
            if kinds == {Isometry3PriorCostTerm}:
                self.terms = PriorTerms(
                    [int(np.asarray(t.entity_indices).reshape(-1)[0]) for t in terms],
                    [t.isometry_prior_mean.params() if isinstance(t.isometry_prior_mean, Isometry3F64)
                     else np.asarray(t.isometry_prior_mean, float) for t in terms],
                    [np.asarray(t.isometry_prior_precision, float) for t in terms])
                return
            if not kinds <= {PinholeCameraReprojectionCostTerm, EucmCameraReprojectionCostTerm} or len(kinds) > 1:
                raise NotOnGpuPath("only PinholeCameraReprojectionCostTerm or EucmCameraReprojectionCostTerm "
                                   "residuals (one kind per CostTerms) run on this backend")
            soa = EucmReprojectionTerms if kinds == {EucmCameraReprojectionCostTerm} else PinholeReprojectionTerms
            self.terms = soa(
                np.array([t.uv_in_image for t in terms], dtype=np.float64).reshape(-1, 2),
                np.array([t.entity_indices for t in terms], dtype=np.int64).reshape(-1, 3))

    @staticmethod
    def new(family_names, terms):
        return CostTerms(family_names, terms)


@dataclass
class HuberKernel:
    delta: float

    @staticmethod
    def new(delta):
        return HuberKernel(float(delta))

    def apply(self, x):
        x = abs(x)
        return x * x if x <= self.delta else 2.0 * self.delta * x - self.delta ** 2

    def weight(self, residual_nrm):
        if residual_nrm == 0.0:
            return 0.0
        return np.sqrt(self.apply(residual_nrm)) / residual_nrm


class RobustKernel:
    @staticmethod
    def Huber(kernel):  # noqa: N802 (mirrors the Rust enum variant)
        return kernel


class CostFn:
    def __init__(self, global_constants, cost_terms, robust_kernel=None):
        self.global_constants = global_constants
        self.cost_terms = cost_terms
        self.robust_kernel = robust_kernel

    @staticmethod
    def new_boxed(global_constants, cost_terms):
        return CostFn(global_constants, cost_terms)

    @staticmethod
    def new_boxed_robust(global_constants, cost_terms, robust_kernel):
        return CostFn(global_constants, cost_terms, robust_kernel)

    def cost_family_names(self):
        return list(self.cost_terms.family_names)


# ---------------------------------------------------------------- params ----
class LinearSolverEnum(enum.Enum):
    DenseLdlt = "DenseLdlt"
    DenseLu = "DenseLu"
    SparseLdlt = "SparseLdlt"
    BlockSparseLdlt = "BlockSparseLdlt"
    FaerSparseQr = "FaerSparseQr"
    FaerSparseLu = "FaerSparseLu"
    FaerSparseLdlt = "FaerSparseLdlt"
    FaerSparseLblt = "FaerSparseLblt"
    SchurBlockSparseLdlt = "SchurBlockSparseLdlt"
    SchurSparseLdlt = "SchurSparseLdlt"
    SchurFaerSparseLdlt = "SchurFaerSparseLdlt"

    def is_schur(self):
        return self.name.startswith("Schur")

    @staticmethod
    def default():
        return LinearSolverEnum.FaerSparseLdlt  # lib.rs:320-324


@dataclass
class OptParams:
    num_iterations: int = 100
    initial_lm_damping: float = 10.0
    parallelize: bool = True
    solver: LinearSolverEnum = field(default_factory=LinearSolverEnum.default)
    skip_final_hessian: bool = False
    function_tolerance: float = 1e-10
    gradient_tolerance: float = 1e-14
    parameter_tolerance: float = 1e-12
    max_consecutive_rejects: int = 20


class TerminationReason(enum.Enum):
    FunctionTolerance = native.TERM_FUNCTION_TOLERANCE
    GradientTolerance = native.TERM_GRADIENT_TOLERANCE
    ParameterTolerance = native.TERM_PARAMETER_TOLERANCE
    MaxIterations = native.TERM_MAX_ITERATIONS
    MaxConsecutiveRejects = native.TERM_MAX_CONSECUTIVE_REJECTS


def _termination(code):
    return None if code == native.TERM_NONE else TerminationReason(code)


@dataclass
class StepInfo:
    merit: float
    smooth_cost: float
    did_outer_step: bool
    inner_step: int
    lm_damping: float
    in_phase1: bool
    termination: Optional[TerminationReason]
    # GB300 diagnostics of the step
    new_merit: float = float("nan")
    gain_ratio: float = float("nan")
    max_step: float = float("nan")
    accepted: bool = False


@dataclass
class OptimizationSolution:
    """OptimizationSolution (crates/sophus_opt/src/nlls/optimizer_types.rs:242-370):
    the variables, the final cost and the steps; covariance_block and
    precision_block answer from the final Hessian on the GPU (built on the
    first query, like the reference's lazily built Covariance)."""
    variables: VarFamilies
    final_cost: float
    steps: List[StepInfo]
    _native: object = field(default=None, repr=False)
    _names: list = field(default=None, repr=False)
    _cov_ready: bool = field(default=False, repr=False)

    def _ref(self, family, idx):
        if self._native is None:
            raise NllsError("this solution holds no final Hessian")
        if family == self._names[0]:
            return (native.VAR_INTRINSICS, int(idx))  # a block only when the camera params are Free
        if family == self._names[1]:
            return (native.VAR_POSE, int(idx))
        if family == self._names[2]:
            return (native.VAR_POINT, int(idx))
        return None  # no such family: None

    def covariance_block(self, row_family, row_var_idx, col_family, col_var_idx):
        """Sigma(i, j): H^-1, or the min-norm H+ for a gauge-deficient H; None
        for a constant variable or an unknown family."""
        row, col = self._ref(row_family, row_var_idx), self._ref(col_family, col_var_idx)
        if row is None or col is None:
            return None
        if not self._cov_ready:
            self._native.covariance_prepare()
            self._cov_ready = True
        return self._native.covariance_block(row, col)

    def precision_block(self, row_family, row_var_idx, col_family, col_var_idx):
        """The block H(i, j) of the undamped final Hessian, or None."""
        row, col = self._ref(row_family, row_var_idx), self._ref(col_family, col_var_idx)
        if row is None or col is None:
            return None
        if not self._cov_ready:
            self._native.covariance_prepare()
            self._cov_ready = True
        return self._native.precision_block(row, col)

    def close(self):
        """Release the device copy of the problem held for the queries."""
        if self._native is not None:
            self._native.close()
            self._native = None


@dataclass
class OptProblem:
    costs: list
    eq_constraints: list = field(default_factory=list)
    ineq_constraints: list = field(default_factory=list)

    @staticmethod
    def costs_only(costs):
        return OptProblem(list(costs))


# ------------------------------------------------------------- dispatch ----
def _validate_solver_config(variables, cost_fns, eq_fns, params):
    """validate_solver_config (crates/sophus_opt/src/nlls/optimizer.rs:649-717)."""
    if eq_fns:
        raise NotOnGpuPath("equality constraints are outside the GPU bundle-adjustment path")
    if not params.solver.is_schur():
        raise NotOnGpuPath("solver %s is not a Schur solver" % params.solver.name)
    nfs = variables.num_free_scalars()
    nms = variables.num_marg_scalars()
    if nfs == 0 or nms == 0:
        raise SchurMissingFreeOrMarg(
            "Schur solver needs free and marginalized variables (free scalars %d, marg scalars %d)" % (nfs, nms))
    for cf in cost_fns:
        marg = [n for n in cf.cost_family_names()
                if n in variables.collection and variables.collection[n].kind == VarKind.Marginalized]
        if len(marg) > 1:
            raise SchurCostConnectsTwoMargFamilies("cost connects %s and %s" % (marg[0], marg[1]))


def _pose_array(members):
    if isinstance(members, np.ndarray):
        return np.ascontiguousarray(members, dtype=np.float64).reshape(-1, 7)
    return np.array([m.params() if isinstance(m, Isometry3F64) else np.asarray(m, float) for m in members],
                    dtype=np.float64).reshape(-1, 7)


def _point_array(members):
    return np.ascontiguousarray(np.asarray(members, dtype=np.float64).reshape(-1, 3))


def _split_costs(cost_fns):
    """The reprojection CostFn and the optional pose-prior CostFn."""
    reproj = [cf for cf in cost_fns if not isinstance(cf.cost_terms.terms, PriorTerms)]
    priors = [cf for cf in cost_fns if isinstance(cf.cost_terms.terms, PriorTerms)]
    if len(reproj) != 1:
        raise NotOnGpuPath("exactly one reprojection CostFn is supported on the GPU path")
    if len(priors) > 1:
        raise NotOnGpuPath("at most one Isometry3PriorCostTerm CostFn is supported on the GPU path")
    for cf in priors:
        if cf.robust_kernel is not None:
            raise NotOnGpuPath("a robust kernel on the pose priors is not on this path")
    return reproj[0], (priors[0] if priors else None)


def _extract_problem(variables, cost_fns):
    cf, prior_cf = _split_costs(cost_fns)
    names = cf.cost_family_names()
    if len(names) != 3:
        raise NotOnGpuPath("reprojection cost needs (intrinsics, pose, point) families")
    fam = [variables.collection[n] for n in names]
    kinds = tuple(f.kind for f in fam)
    if kinds not in ((VarKind.Conditioned, VarKind.Free, VarKind.Marginalized),
                     (VarKind.Free, VarKind.Free, VarKind.Marginalized)):
        raise NotOnGpuPath("GPU path needs kinds (Conditioned or Free, Free, Marginalized), got %s" % (kinds,))
    if kinds[0] == VarKind.Free and fam[0].constant_ids:
        raise NotOnGpuPath("a constant id in a Free intrinsics family is not on this path")
    intr = fam[0].members
    if len(intr) != 1:
        raise NotOnGpuPath("GPU path supports one intrinsics member")
    cam = intr[0]
    terms = cf.cost_terms.terms
    eucm = isinstance(terms, EucmReprojectionTerms)
    if eucm != isinstance(cam, EnhancedUnifiedCameraF64) and not isinstance(cam, np.ndarray):
        raise NotOnGpuPath("the camera type does not match the reprojection cost term")
    cparams = cam.params if isinstance(cam, (PinholeCameraF64, EnhancedUnifiedCameraF64)) else np.asarray(cam, float)
    if cparams.size != (6 if eucm else 4):
        raise NotOnGpuPath("camera params: expected %d, got %d" % (6 if eucm else 4, cparams.size))
    idx = terms.entity_indices
    if idx.shape[0] and (idx[:, 0].min() < 0 or idx[:, 0].max() != 0):
        raise NotOnGpuPath("intrinsics index must be 0")
    poses = _pose_array(fam[1].members)
    points = _point_array(fam[2].members)
    pc = np.zeros(poses.shape[0], np.uint8)
    for i in fam[1].constant_ids:
        pc[i] = 1
    qc = None
    if fam[2].constant_ids:
        qc = np.zeros(points.shape[0], np.uint8)
        for i in fam[2].constant_ids:
            qc[i] = 1
    huber = cf.robust_kernel.delta if cf.robust_kernel is not None else 0.0
    prob = BAProblem(poses=poses, points=points, intrinsics=np.asarray(cparams[:4], float),
                     obs_cam=idx[:, 1].astype(np.int32), obs_pt=idx[:, 2].astype(np.int32),
                     obs_uv=terms.uv_in_image, huber_delta=huber, pose_const=pc, point_const=qc)
    prob.intrinsics_free = kinds[0] == VarKind.Free
    if eucm:
        prob.camera_model = native.CAMERA_EUCM
        prob.eucm_alpha_beta = np.asarray(cparams[4:6], float).copy()
    prob.priors = None
    if prior_cf is not None:
        if prior_cf.cost_family_names() != [names[1]]:
            raise NotOnGpuPath("the pose priors must act on the reprojection cost's pose family")
        prob.priors = prior_cf.cost_terms.terms
    return prob, names


def _set_priors(gp, prob):
    if getattr(prob, "priors", None) is not None:
        t = prob.priors
        gp.set_pose_priors(t.pose, t.mean, t.precision)


def _step_info(rec, k):
    return StepInfo(merit=rec.merit, smooth_cost=rec.merit, did_outer_step=False, inner_step=k,
                    lm_damping=rec.lm_damping, in_phase1=False, termination=_termination(rec.termination),
                    new_merit=rec.new_merit, gain_ratio=rec.gain_ratio, max_step=rec.max_step,
                    accepted=bool(rec.accepted))


def _write_back(variables, names, poses, points, intrinsics=None):
    fams = dict(variables.collection)
    if intrinsics is not None:
        cf = fams[names[0]]
        cam = cf.members[0]
        if isinstance(cam, (PinholeCameraF64, EnhancedUnifiedCameraF64)):
            new = type(cam)(np.asarray(intrinsics, float), cam.image_size)
        else:
            new = np.asarray(intrinsics, float)
        fams[names[0]] = VarFamily(cf.kind, [new], sorted(cf.constant_ids))
    pf = fams[names[1]]
    if isinstance(pf.members, np.ndarray):
        pm = poses.copy()
    else:
        pm = [Isometry3F64(p) for p in poses]
    fams[names[1]] = VarFamily(pf.kind, pm, sorted(pf.constant_ids))
    qf = fams[names[2]]
    qm = points.copy() if isinstance(qf.members, np.ndarray) else [p.copy() for p in points]
    fams[names[2]] = VarFamily(qf.kind, qm, sorted(qf.constant_ids))
    return VarFamilies(fams)


class Optimizer:
    """Stateful LM optimizer on the GPU (Optimizer::new / step / build_solution)."""

    def __init__(self, variables, problem, params, device=-1):
        costs = problem.costs if isinstance(problem, OptProblem) else list(problem)
        eq = problem.eq_constraints if isinstance(problem, OptProblem) else []
        if isinstance(problem, OptProblem) and problem.ineq_constraints:
            raise NotOnGpuPath("inequality constraints are outside the GPU bundle-adjustment path")
        _validate_solver_config(variables, costs, eq, params)
        prob, names = _extract_problem(variables, costs)
        self._variables = variables
        self._names = names
        self._params = params
        self._gpu = native.Problem(prob, device=device)
        _set_priors(self._gpu, prob)
        self._gpu.init(params)
        self._steps = []

    @staticmethod
    def new(variables, problem, params):
        return Optimizer(variables, problem, params)

    def step(self):
        rec = self._gpu.step()
        info = _step_info(rec, len(self._steps))
        self._steps.append(info)
        return info

    def _intrinsics(self):
        return self._gpu.intrinsics() if self._variables.collection[self._names[0]].kind == VarKind.Free else None

    def variables(self):
        poses, points = self._gpu.variables()
        return _write_back(self._variables, self._names, poses, points, self._intrinsics())

    def build_solution(self):
        poses, points = self._gpu.variables()
        cost = self._gpu.cost()
        # the device problem moves to the solution (covariance / precision queries)
        sol = OptimizationSolution(_write_back(self._variables, self._names, poses, points, self._intrinsics()),
                                   cost, self._steps, self._gpu, list(self._names))
        self._gpu = None
        return sol


def optimize_nlls(variables, cost_fns, eq_fns, params, device=-1):
    """optimize_nlls on the GPU: steps until a termination reason, then build_solution."""
    _validate_solver_config(variables, cost_fns, eq_fns, params)
    prob, names = _extract_problem(variables, cost_fns)
    gp = native.Problem(prob, device=device)
    try:
        _set_priors(gp, prob)
        recs, _ = gp.optimize(params)
        poses, points = gp.variables()
        intr = gp.intrinsics() if prob.intrinsics_free else None
        cost = gp.cost()
    except BaseException:
        gp.close()
        raise
    steps = [_step_info(r, k) for k, r in enumerate(recs)]
    # the device problem stays with the solution for covariance / precision queries
    return OptimizationSolution(_write_back(variables, names, poses, points, intr), cost, steps, gp, list(names))
