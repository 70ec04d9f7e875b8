"""galax_gb300: the orbit-integration hot path of GalacticDynamics/galax on GB300.

Potentials (``galax_gb300.potential``) and orbit integration
(``galax_gb300.dynamics``) with galax's interface, run by a CUDA library for
sm_103a through the C ABI in ``include/galax_gb300.h``. There is no CPU path:
without the built library or a CUDA device, calls raise.
"""

from . import dynamics, mockstream, potential
from ._lib import GalaxGB300Error
from .dynamics import (
    ConstantStepSize,
    Dopri5,
    Dopri8,
    HamiltonianField,
    Integrator,
    Orbit,
    OrbitSolver,
    PhaseSpaceCoordinate,
    PIDController,
    compute_orbit,
    evaluate_orbit,
    integrate_orbit,
)
from .mockstream import ChenStreamDF, Fardal2015DF, FardalStreamDF, MockStreamGenerator, StreamSimulator
from .potential import (
    BovyMWPotential2014,
    CompositePotential,
    HernquistPotential,
    IsochronePotential,
    KeplerPotential,
    LinearParameter,
    LogarithmicPotential,
    MilkyWayPotential,
    MilkyWayPotential2022,
    MiyamotoNagaiPotential,
    MN3ExponentialPotential,
    MN3Sech2Potential,
    NFWPotential,
    PlummerPotential,
    PowerLawCutoffPotential,
    TranslatedPotential,
)

__all__ = [
    "GalaxGB300Error", "dynamics", "mockstream", "potential", "ConstantStepSize", "Dopri5", "Dopri8", "Integrator",
    "Orbit", "OrbitSolver", "PhaseSpaceCoordinate", "PIDController", "compute_orbit", "evaluate_orbit", "HamiltonianField", "integrate_orbit",
    "ChenStreamDF", "Fardal2015DF", "FardalStreamDF", "MockStreamGenerator", "StreamSimulator",
    "BovyMWPotential2014", "CompositePotential", "HernquistPotential", "IsochronePotential", "KeplerPotential", "LinearParameter", "LogarithmicPotential",
    "MilkyWayPotential", "MilkyWayPotential2022", "MiyamotoNagaiPotential", "MN3ExponentialPotential",
    "MN3Sech2Potential", "NFWPotential", "PlummerPotential", "PowerLawCutoffPotential", "TranslatedPotential",
]
