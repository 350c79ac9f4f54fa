"""qbgpu — GB300-native boundary-integral hot path of QuantumBilliards.jl.

Host-side mirror of the reference's operator API for the path (geometry,
workspaces, assembly, Beyn contour step, sigma_min sweep) over the C ABI of
libqbgpu.so. Import fails if the library has not been built.
"""
from . import _lib
from .geometry import (BoundaryPointsCFIE, make_circle, make_star, make_full_stadium, make_circle_with_hole,
                       make_rectangle, make_full_ellipse_mushroom, multi_kress_graded_nodes_data,
                       s_mid)
from .solvers import (DLP_kress, DLP_kress_global_corners, CFIE_kress, CFIE_kress_global_corners, CFIE_alpert,
                      evaluate_points, points_with_n)
from . import operators
from .operators import (Workspace, build_workspace, assemble, assemble_noalloc, construct_matrices,
                        construct_boundary_matrices,
                        construct_boundary_matrices_with_derivatives, bessel01, sigma_min, cgemm,
                        set_gemm_engine, launch_count, chebyshev_params, residual_c64, zgemm_sub_tc,
                        release_cached_memory, pool_stats, adjoint_fredholm_matrix, solve_vect_dlp,
                        chebyshev_params_min_cost)
from .beyn import BeynHandle, construct_B_matrix, solve_vect, solve, solve_disks, solve_pipelined, probe_matrix, contour
from .sweep import k_sweep, get_eigenvalues, newton_refine_svd, refine_minima
from . import sweep
from . import ebim
from . import autotune
from .serve import Server
from .spectrum import (plan_weyl_windows, beyn_disks_from_windows, candidate_residuals,
                       residual_and_norm_select, imag_k_check, compute_spectrum_beyn)
from .symmetry import (Reflection, Rotation, XReflection, YReflection, XYReflection,
                       periodic_symmetry_index_orbits)

_lib.load()

__all__ = [n for n in dir() if not n.startswith("_")]
