"""Initial ion state sampled on the device (od_init_state) against the distributions of
opendust.py:373-451: uniform in the cylinder outside every grain; N(0, v_T) across and
N(v_fl, v_T) along the axis (Maxwellian) or the tabulated field-driven v_z. Statistical bounds
are 5 standard errors."""
import numpy as np
import pytest

from opendust_gb300 import _lib, setup_host, workloads
from tests._util import case

pytestmark = pytest.mark.gpu


def test_device_initial_state_maxwellian(gpu_lib):
    N = 2**16
    holder, _, _, plasma, sim, grains = case(N=N, n=4, seed=51)
    with _lib.Engine(holder) as eng:
        eng.init_state()
        pos, vel = eng.get_state()
        eng.step(2)
    lam = plasma.r_D_e
    rho2 = pos[:, 0] ** 2 + pos[:, 1] ** 2
    assert np.all(rho2 <= (sim.R * (1 + 1e-6)) ** 2) and np.all(np.abs(pos[:, 2]) <= sim.H / 2 * (1 + 1e-6))
    g = grains[0]
    d = np.linalg.norm(pos - np.array([g.x, g.y, g.z]), axis=1)
    assert np.all(d > g.r * (1 - 1e-5))
    se = lambda s: 5 * s / np.sqrt(N)
    assert abs(rho2.mean() - sim.R**2 / 2) < se(sim.R**2 / np.sqrt(12))
    assert abs(pos[:, 2].mean()) < se(sim.H / np.sqrt(12))
    for k, mu in ((0, 0.0), (1, 0.0), (2, plasma.v_fl)):
        assert abs(vel[:, k].mean() - mu) < se(plasma.v_T)
        assert abs(vel[:, k].std() / plasma.v_T - 1) < 0.02
    assert lam > 0


def test_device_initial_state_field_driven(gpu_lib):
    N = 2**16
    holder, _, _, plasma, sim, grains = case(N=N, n=4, seed=52, builder=workloads.field_chain)
    v, xi = setup_host.field_driven_vz_table(plasma.v_fl, plasma.v_T)
    with _lib.Engine(holder) as eng:
        eng.init_state((v, xi))
        pos, vel = eng.get_state()
    # mean of the tabulated distribution (piecewise-linear inverse CDF)
    mean = np.sum(0.5 * (v[1:] + v[:-1]) * np.diff(xi))
    sd = np.sqrt(np.sum(0.5 * (v[1:] ** 2 + v[:-1] ** 2) * np.diff(xi)) - mean**2)
    assert abs(vel[:, 2].mean() - mean) < 5 * sd / np.sqrt(N)
    for g in grains:
        d = np.linalg.norm(pos - np.array([g.x, g.y, g.z]), axis=1)
        assert np.all(d > g.r * (1 - 1e-5))
