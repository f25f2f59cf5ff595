"""deo -- DiffEqOperators.jl's stencil-apply path on GB300 (sm_103a).

The public names mirror the reference package (CenteredDifference,
UpwindDifference, RobinBC, GeneralBC, DirichletBC, Dirichlet0BC, NeumannBC,
Neumann0BC, PeriodicBC, MultiDimBC, compose, `L*Q*u`, mul!) and run on the
CUDA kernels of libdeo.so.  There is no CPU fallback.
"""
from ._lib import (DEO_OPT_CONCURRENT_SHELL, DEO_OPT_EXACT_SUMS, DEO_OPT_FAST_PATH, DEO_OPT_FX_FP64_ROWS, DEO_OPT_LAUNCH_TIMING, DEO_OPT_TEST_WITHHOLD, DEO_OPT_F32_VECTOR, DEO_OPT_SHELL_KERNEL, DEO_OPT_F32_TILE, DEO_OPT_TMA, DeoArgError, DeoError,  # noqa: F401
                   DEO_PLAN_FACTOR_FIELD, DEO_PLAN_MERGE_TERMS, DEO_PLAN_STAR, DeoShapeError, LIB_PATH, lib)


def device_status() -> int:
    """Device-side error flags since the last call (bit 0: a bounded wait gave up)."""
    import ctypes
    v = ctypes.c_uint(0)
    lib().deo_device_status(ctypes.byref(v))
    return v.value
from .operators import (  # noqa: F401
    AtomicBC, CenteredDifference, ComposedMultiDimBC, DerivativeOperator, DiffEqOperatorCombination,
    DimensionMismatch, Dirichlet0BC, DirichletBC, FieldCoefficient, GeneralBC, GhostDerivativeOperator,
    MultiDimBC, MultiDimDirectionalBC, Neumann0BC, NeumannBC, PeriodicBC, Plan, RobinBC, UpwindDifference,
    calculate_weights, clear_plan_cache, compose, concretize, fortran_strides, julia_array, ldiv, ldiv_, mul_,
    operator_from_tables, plan_for, SolvePlan, solve_plan_for, to_julia_layout, with_field,
)

mul = mul_
from . import autodiff, batch  # noqa: E402,F401
from .autodiff import rrule  # noqa: E402,F401
from .batch import Batch, StageBatch  # noqa: E402,F401
from .nonlinear import nonlinear_diffusion, nonlinear_diffusion_  # noqa: E402,F401
from .vector import (Curl, CurlOperator, Divergence, DivergenceOperator, Gradient, GradientOperator,  # noqa: E402,F401
                     cross_product, cross_product_, dot_product, dot_product_, square_norm, square_norm_)
