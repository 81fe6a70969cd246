"""`opendust.opendust` module path of the reference, backed by opendust_gb300."""
from opendust_gb300.opendust import *  # noqa: F401,F403
from opendust_gb300.opendust import (  # noqa: F401
    DustParticle,
    OpenDust,
    OutputParameters,
    PlasmaParametersInSIUnitsFieldDriven,
    PlasmaParametersInSIUnitsMaxwell,
    SimulatioParametersInSIUnits,
    SimulationParametersInSIUnits,
)
