"""GB300-native superion step engine with OpenDust's Python API."""
from .opendust import (  # noqa: F401
    DustParticle,
    OpenDust,
    OutputParameters,
    PlasmaParametersInSIUnitsFieldDriven,
    PlasmaParametersInSIUnitsMaxwell,
    SimulatioParametersInSIUnits,
    SimulationParametersInSIUnits,
    build_simulation,
)

__version__ = "0.1.0"
