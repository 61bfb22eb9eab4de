"""The engine under the module name the reference's README and examples use
(``pibronic.pimc.minimal``, e.g. examples/basic_ml_testing.py:17): the same objects as
``pibronic_gb300.pimc``."""
from .pimc import *  # noqa: F401,F403
from .pimc import (__all__ as _pimc_all, build_denominator, build_numerator, build_o_matrix,  # noqa: F401
                   build_scaling_factors, block_compute_gR, block_compute_gR_from_raw_samples,
                   block_compute_rhoR_from_input_samples, diagonalize_coupling_matrix,
                   save_gR_with_samples, scale_o_matrices)

__all__ = list(_pimc_all) + ["build_o_matrix", "build_scaling_factors", "scale_o_matrices",
                             "build_denominator", "diagonalize_coupling_matrix", "build_numerator",
                             "block_compute_gR", "save_gR_with_samples",
                             "block_compute_gR_from_raw_samples", "block_compute_rhoR_from_input_samples"]
