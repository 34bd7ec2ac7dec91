"""GB300-native explicit time marching for BristolFE-v2 models.

The compute path is the native library ``libbfe_gb300.so`` (hand-written
sm_103a kernels behind the C ABI in ``include/bfe_gb300.h``); this package is
its host-side mirror of the reference's solver interface.
"""
from ._lib import BfeError, load  # noqa: F401
from .field import FieldOutput, fn_get_field_output_gb300  # noqa: F401
from .assembly import DeviceMatrices, assemble_gpu  # noqa: F401
from .fmc import (fn_convert_disps_to_forces_v2_gb300, fn_convolve_gb300,  # noqa: F401
                  fn_parse_to_fmc_gb300)
from .solver import (V5, VEL_CURRENT, VEL_LAST_HALF, Plan, SolverError,  # noqa: F401
                     fn_explicit_dynamic_solver_gb300, fn_explicit_dynamic_solver_v5_gb300)

__version__ = "0.1.0"
