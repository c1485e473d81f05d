"""omega3d_gb300: GB300 (sm_103a) Biot-Savart velocity/gradient and BEM hot path of
Omega3D behind a C-ABI (include/o3dgpu.h, libo3dgpu.so) with a reference-shaped
Python mirror of its call surface."""
from ._lib import CORES, PRECS, O3GError, lib, header_symbols  # noqa: F401
from .influence import (BEM, Batch, BatchRalston, BatchSystem, ExecEnv, Ralston, InfluenceVisitor, Points,  # noqa: F401
                        ResultsType, Surfaces, clear_inner_layer, device_matrix_view, merge_close_particles, represent_as_particles,
                        shed_particles, split_elongated,
                        generate_ovoid, panels_affect_panels, panels_affect_points, panels_on_panels_coeff,
                        points_affect_panels,
                        points_affect_points, solve_bem)

__all__ = ["CORES", "PRECS", "O3GError", "lib", "header_symbols", "ExecEnv", "InfluenceVisitor", "Points",
           "ResultsType", "points_affect_points", "Surfaces", "generate_ovoid", "panels_affect_points",
           "panels_affect_panels",
           "points_affect_panels", "panels_on_panels_coeff", "BEM", "solve_bem", "Ralston", "Batch",
           "BatchSystem", "BatchRalston", "clear_inner_layer",
           "represent_as_particles", "split_elongated", "merge_close_particles", "shed_particles",
           "device_matrix_view"]
