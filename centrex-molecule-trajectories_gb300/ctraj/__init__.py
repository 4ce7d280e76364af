"""ctraj -- GB300-native engine for the molecular-beam trajectory hot path.

Drop-in for ``trajectories.trajectory_simulator.TrajectorySimulator`` of
otimgren/centrex-molecule-trajectories: the same Beamline / BeamlineElement /
Distribution / Counter API, with propagation done by hand-written sm_103a
CUDA kernels in ``libctraj.so`` behind the C ABI in ``include/ctraj.h``.
"""
from .beamline import Beamline
from .beamline_elements import (CircularAperture, ElectrostaticLens, FieldPlates, Honeycomb,
                                RectangularAperture)
from .distributions import (CeNTREXPositionDistribution, CeNTREXVelocityDistribution,
                            GaussianDistribution, GaussianPositionDistribution)
from .molecule import Molecule, Trajectory
from .stark import StarkForce, TwoLevelStark, hexapole_force, reference_radial_table
from .trajectory_simulator import Counter, SimulationResult, TrajectorySimulator

__all__ = [
    "Beamline", "CircularAperture", "RectangularAperture", "FieldPlates", "ElectrostaticLens", "Honeycomb",
    "GaussianDistribution", "CeNTREXVelocityDistribution", "CeNTREXPositionDistribution",
    "GaussianPositionDistribution", "Molecule", "Trajectory", "StarkForce", "TwoLevelStark",
    "hexapole_force", "reference_radial_table", "TrajectorySimulator", "Counter", "SimulationResult",
]
