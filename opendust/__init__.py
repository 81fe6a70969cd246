"""Import-compatible shim: `from opendust import X` and `from opendust.opendust import X`
resolve to the GB300 engine's classes (the reference's package layout)."""
from opendust_gb300.opendust import (  # noqa: F401
    DustParticle,
    OpenDust,
    OutputParameters,
    PlasmaParametersInSIUnitsFieldDriven,
    PlasmaParametersInSIUnitsMaxwell,
    SimulatioParametersInSIUnits,
    SimulationParametersInSIUnits,
)
from . import opendust  # noqa: F401,E402
