"""Reference-layout import path for the chains/matthews.py fork: ``from opendust.matthews import
OpenDust, PlasmaParametersInSIUnitsMatthews, ...`` (the reference scripts put chains/ on sys.path
and ``import matthews``)."""
from opendust_gb300.matthews import (  # noqa: F401
    DustDynamics,
    DustParticle,
    OpenDust,
    OutputParameters,
    PlasmaParametersInSIUnitsMatthews,
    SimulatioParametersInSIUnits,
    SimulationParametersInSIUnits,
)
