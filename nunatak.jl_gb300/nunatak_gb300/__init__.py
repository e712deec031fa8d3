"""nunatak_gb300 — GB300-native velocity solve of Nunatak.jl (SSA / DIVA Picard + PCG) behind a C ABI.

The compute path is libnunatak_gb300.so (hand-written CUDA for sm_103a); this package is the host-side
mirror of the reference's configuration objects and solver entry points."""
from . import abi
from .model import (YEAR, Convergence, DepthIntegrated, DIVAShear, FixedIterations, FreeSlipWalls, GlenFlowLaw,
                    IceSheetConstants, LineJacobi, NoSlipWalls, PointJacobi, RectilinearGrid,
                    RegularizedCoulombFriction, SmoothIceMask, StressBalanceDiagonalPreconditioner,
                    StressBalanceMultigridPreconditioner, StressBalanceSolver, SubgridGroundedFraction,
                    UpwindBiased, ViscosityConvergence, WENO, WeertmanFriction, default_thickness_advection,
                    PartialCellFront, ThicknessThresholdCalving, EigenCalving, VonMisesCalving, FrontVelocityCalving,
                    MaximumExtentCalving, TillEffectivePressure,
                    make_descriptors, field_shape, sigma_faces)
from .problem import NunatakError, Problem
from .batch import Batch

__all__ = [
    "abi", "YEAR", "Convergence", "DepthIntegrated", "DIVAShear", "FixedIterations", "FreeSlipWalls", "GlenFlowLaw",
    "IceSheetConstants", "LineJacobi", "NoSlipWalls", "PointJacobi", "RectilinearGrid", "RegularizedCoulombFriction",
    "SmoothIceMask", "StressBalanceDiagonalPreconditioner", "StressBalanceMultigridPreconditioner",
    "StressBalanceSolver", "SubgridGroundedFraction", "ViscosityConvergence", "WeertmanFriction", "make_descriptors",
    "field_shape", "sigma_faces", "UpwindBiased", "WENO", "default_thickness_advection", "PartialCellFront",
    "ThicknessThresholdCalving", "EigenCalving", "VonMisesCalving", "FrontVelocityCalving", "MaximumExtentCalving",
    "TillEffectivePressure", "NunatakError", "Problem", "Batch",
]
