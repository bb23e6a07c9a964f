"""GB300-native dense 2-D BEM collocation path (assemble -> applyBC -> solve)."""
import os as _os

# The batched solves overlap up to 32 worker streams; the CUDA driver maps
# streams to hardware work queues, 8 unless this is set before the first CUDA
# call of the process (an explicit setting is kept).
_os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
from .geometry import (BEMdata, Laplace, Elasticity, quadrado, quadrado_elasticity, star_domain,
                       plate_with_hole, ana_laplace_linear, ana_laplace_expcos,
                       ana_elasticity_patch, attach_analytical, apply_analytical_bc, rel_error,
                       rel_error_flux, from_cad, from_nodes, star_adjoint_case, internal_grid,
                       point_in_domain, format2d)
