"""GB300 (sm_103a) backend for the weakly-compressible SPH right-hand side of TrixiParticles.jl.

The compute path is libtp_wcsph.so (CUDA C++ behind the C ABI of include/tp_wcsph.h); this
package is the host-side mirror of the reference's drop-in surface (Semidiscretization,
semidiscretize, kick!/drift!, solve with CarpenterKennedy2N54) plus the dam-break setup.
"""
from ._abi import TpConfig, TpError, default_config, load_library
from .build import build
from .semidiscretization import (
    AdamiPressureExtrapolation,
    ArtificialViscosityMonaghan,
    BoundaryModelDummyParticles,
    CarpenterKennedy2N54,
    ContinuityDensity,
    DensityDiffusionMolteniColagrossi,
    FullGridCellList,
    GB300Backend,
    GridNeighborhoodSearch,
    ODEProblem,
    Semidiscretization,
    CallbackSet,
    InfoCallback,
    SortingCallback,
    StepsizeCallback,
    SymplecticPositionVerlet,
    WallBoundarySystem,
    WeaklyCompressibleSPHSystem,
    WendlandC2Kernel,
    dam_break_semidiscretization,
    drift,
    kick,
    semidiscretize,
    solve,
)
from .setups import InitialCondition, RectangularShape, RectangularTank, StateEquationCole, \
    dam_break
from . import adjoint, ensemble, interpolation, vtk
from .vtk import SolutionSavingCallback, trixi2vtk, vtk2trixi
from .interpolation import interpolate_line, interpolate_plane_2d, interpolate_plane_3d, \
    interpolate_points

__all__ = [
    "AdamiPressureExtrapolation", "ArtificialViscosityMonaghan", "BoundaryModelDummyParticles",
    "CarpenterKennedy2N54", "ContinuityDensity", "DensityDiffusionMolteniColagrossi",
    "FullGridCellList", "GB300Backend", "GridNeighborhoodSearch", "InitialCondition",
    "ODEProblem", "RectangularShape", "RectangularTank", "Semidiscretization", "StateEquationCole",
    "SortingCallback", "StepsizeCallback", "CallbackSet", "InfoCallback", "SymplecticPositionVerlet", "TpConfig",
    "TpError", "WallBoundarySystem", "WeaklyCompressibleSPHSystem", "WendlandC2Kernel",
    "SolutionSavingCallback", "adjoint", "build", "dam_break", "ensemble", "trixi2vtk",
    "vtk", "vtk2trixi", "interpolate_line", "interpolate_points", "interpolate_plane_2d",
    "interpolate_plane_3d",
    "interpolation", "dam_break_semidiscretization", "default_config", "drift", "kick",
    "load_library", "semidiscretize", "solve",
]
