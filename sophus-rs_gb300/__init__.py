"""GB300-native Schur-complement Levenberg-Marquardt bundle adjustment.

A drop-in backend for sophus-rs's optimize_nlls on the bundle-adjustment
path.  The compute is libsgba.so (hand-written sm_103a CUDA kernels behind the
C ABI in include/sgba.h); this package is its Python mirror of the sophus_opt
API plus the seeded synthetic scene generator.
"""
from . import native, synth  # noqa: F401
from .opt import (  # noqa: F401
    CostFn,
    CostTerms,
    EnhancedUnifiedCameraF64,
    EucmCameraReprojectionCostTerm,
    EucmReprojectionTerms,
    HuberKernel,
    Isometry3F64,
    Isometry3PriorCostTerm,
    LinearSolverEnum,
    LinearSolverError,
    NllsError,
    NotOnGpuPath,
    OptimizationSolution,
    Optimizer,
    OptParams,
    OptProblem,
    PinholeCameraF64,
    PinholeCameraReprojectionCostTerm,
    PinholeReprojectionTerms,
    PriorTerms,
    RobustKernel,
    SchurCostConnectsTwoMargFamilies,
    SchurMissingFreeOrMarg,
    SolverDoesNotSupportEqConstraints,
    StepInfo,
    TerminationReason,
    VarBuilder,
    VarFamilies,
    VarFamily,
    VarKind,
    optimize_nlls,
)
from .synth import BAProblem  # noqa: F401
