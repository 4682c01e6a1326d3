"""jaxtrace_gb300 -- GB300-native Lagrangian particle tracking.

A drop-in for JAXTrace's tracking hot path: ``create_tracker(...)
.track_particles()`` with the same field / integrator / boundary / density
signatures and ``Trajectory`` layout, running hand-written sm_103a CUDA
kernels through the C ABI in ``include/jaxtrace_gb300.h``.
"""
from .boundary import (absorbing_boundary_factory, clamping_boundary, continuous_inlet_boundary_factory,
                       mixed_boundary, no_boundary, periodic_boundary, reflective_boundary, unit_box_periodic,
                       unit_box_reflective, clamp_to_bounds, reflect_boundary)
from .fields import (FEMTimeSeriesField, FemHashGrid, OctreeFEMTimeSeriesFieldOptimized, OctreeMesh, StructuredGridSampler,
                     StructuredTimeSeriesField, TimeSeriesField)
from .integrators import euler_step, rk2_step, rk4_step
from .particles import (Trajectory, compute_trajectory_statistics, create_empty_trajectory,
                        create_single_particle_trajectory, create_trajectory_from_positions, merge_trajectories,
                        validate_trajectory_data)
from .analysis import analyze_trajectory_results, compute_mixing_metrics
from .density import KDEEstimator, SPHDensityEstimator
from .seeding import random_seeds, uniform_grid_seeds
from .tracker import (EnsembleBatch, ParticleTracker, TrackerOptions, compare_integrators, create_tracker,
                      track_particles_simple)
from .autotune import Autotuner
from .vtk_io import (VTKTrajectorySeries, VTKTrajectoryWriter, VTKUnstructuredTimeSeriesReader,
                     create_field_from_vtk, create_time_series_from_vtk_files, open_dataset, open_vtk_time_series)
from .fields import TimeDependentVelocityField, TimeVaryingField

__version__ = "0.1.0"

__all__ = [
    "TimeSeriesField", "StructuredGridSampler", "StructuredTimeSeriesField", "OctreeFEMTimeSeriesFieldOptimized",
    "OctreeMesh", "euler_step", "rk2_step", "rk4_step", "Trajectory", "ParticleTracker", "TrackerOptions",
    "create_tracker", "track_particles_simple", "random_seeds", "uniform_grid_seeds", "periodic_boundary",
    "reflective_boundary", "clamping_boundary", "absorbing_boundary_factory", "mixed_boundary",
    "continuous_inlet_boundary_factory", "no_boundary", "unit_box_periodic", "unit_box_reflective",
    "EnsembleBatch", "Autotuner", "FEMTimeSeriesField", "FemHashGrid", "compute_trajectory_statistics",
    "compute_mixing_metrics", "VTKTrajectoryWriter", "VTKTrajectorySeries", "VTKUnstructuredTimeSeriesReader",
    "open_vtk_time_series", "create_trajectory_from_positions", "create_single_particle_trajectory",
    "create_empty_trajectory", "merge_trajectories", "validate_trajectory_data", "compare_integrators",
    "analyze_trajectory_results", "KDEEstimator", "SPHDensityEstimator", "clamp_to_bounds", "reflect_boundary",
    "open_dataset", "create_field_from_vtk", "create_time_series_from_vtk_files", "TimeDependentVelocityField",
    "TimeVaryingField",
]
