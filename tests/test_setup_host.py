"""Host setup (opendust_gb300/setup_host.py) on the CPU: the trap-fit grid and least squares
(opendust.py:499-550) recover a known polynomial, and the field-driven initial v_z table is a
proper CDF with the distribution's mean drift."""
import numpy as np
import pytest

from opendust_gb300 import setup_host as sh


def test_trap_grid_matches_reference_formulas():
    lam = 1.1754e-3
    Rh, Hh, n_r, n_h, n_points = sh.trap_grid(3 * lam, 6 * lam, lam)
    assert Rh == pytest.approx(3.0) and Hh == pytest.approx(6.0)
    assert (n_r, n_h) == (int(Rh * 10), int(Hh * 5))
    assert n_points == int(np.pi * Rh**2 * Hh / 0.05**3)


def test_fit_trap_recovers_polynomial():
    Rh, Hh, N = 3.0, 6.0, 4096
    n_r, n_h = int(Rh * 10), int(Hh * 5)
    rng = np.random.default_rng(0)
    coef = rng.normal(0, 1, 15) * np.logspace(0, -6, 15)
    A = sh.trap_design_matrix(np.linspace(0, Rh, n_r), np.linspace(0, Hh / 2, n_h))
    pot = (A @ coef).reshape(n_r, n_h)
    alpha = sh.fit_trap(pot, Rh, Hh, N)
    np.testing.assert_allclose(alpha, -coef * N, rtol=1e-6, atol=1e-9 * N)


def test_field_driven_vz_table_is_a_cdf():
    v_fl, v_T = 1200.0, 250.0
    v, xi = sh.field_driven_vz_table(v_fl, v_T)
    assert xi[0] == 0.0 and xi[-1] == pytest.approx(1.0, abs=1e-9)
    assert np.all(np.diff(xi) >= -1e-15) and np.all(np.diff(v) > 0)
    # samples through the inverse CDF drift downstream at a speed of the order of v_fl
    u = np.random.default_rng(1).uniform(0, 1, 200000)
    vz = sh.field_driven_vz(v_fl, v_T, u)
    assert np.all(np.isfinite(vz)) and v.min() <= vz.min() and vz.max() <= v.max()
    assert 0.5 * v_fl < vz.mean() < 2.0 * v_fl


def _tab_eval(v, xi, sl, u):
    # the device's and the oracle's lookup (first node at or above u, linear from the one before)
    i = 1
    while i < len(v) - 1 and u > xi[i]:
        i += 1
    return v[i - 1] + (u - xi[i - 1]) * sl[i]


def test_injection_tables_finite_at_every_draw():
    # a slow field-driven flow (Mach 0.02: the test_gpu_api plasma) leaves the side v_z CDF flat
    # (0 to double precision) over its leading nodes, as fast flows can for the face fluxes;
    # draws of exactly 0 and 1 must still give finite speeds
    for M in (0.0196582722, 1.0, 2.0):
        v_T = 249.87926383157722
        for dist in ("Maxwellian", "fieldDriven"):
            tables, probs = sh.injection_setup(M * 2457.3, v_T, 3e-3, 6e-3, dist)
            for v, xi, sl in tables:
                v, xi, sl = (np.asarray(a, dtype=np.float64) for a in (v, xi, sl))
                if len(v) == 0:
                    continue
                assert np.all(np.isfinite(sl)), (M, dist)
                for u in (0.0, 2.0**-24, 0.5, 1.0 - 2.0**-24, 1.0):
                    assert np.isfinite(_tab_eval(v, xi, sl, u)), (M, dist, u)
