"""CPU tests of the chains/matthews.py fork model: the oracle's tabulated trap (natural cubic
splines, against scipy), the order-2 field, the top-face re-injection and side-wall reflection
of one step, the per-height trap fit, the trap file and the out-of-domain factor."""
import numpy as np
import pytest
from scipy.interpolate import CubicSpline

from opendust_gb300 import matthews as mt
from opendust_gb300 import setup_host as sh
from oracle import oracle


def fork_case(N=4, order=2, n=4, grains=None, w_c=0.0, table=None, M=1.0):
    """A small fork configuration (launch.py-like plasma, R = 1.25, H = 5 r_D_e)."""
    E_0 = 2600.0
    phi = {"E_0": [E_0, "V/m"], "alpha": [2.4e6, "V/m^2"], "beta": [3.0e8, "V/m^3"],
           "z1": [-1.0e-3, "m"], "z7": [1.5e-3, "m"]}
    plasma = mt.PlasmaParametersInSIUnitsMatthews(290.0, 30000.0, 1e14, order, phi, M, w_c,
                                                  6.6335209e-26)
    lam = plasma.r_D_e
    sim = mt.SimulatioParametersInSIUnits(1.25 * lam, 5 * lam, N, n, 1e-9, plasma)
    if grains is None:
        grains = [mt.DustParticle(0.0, 0.0, -0.5 * lam, 4.4e-6, "consistent", -1e-15),
                  mt.DustParticle(0.0, 0.0, 0.5 * lam, 4.4e-6, "given", -2e-15)]
    holder = mt.build_matthews(plasma, sim, grains, trap_table=table, consider_trap=table is not None)
    return holder, plasma, sim, grains


def smooth_table(n=50):
    h = np.linspace(-2.5, 2.5, n)
    return np.vstack([0.3 * np.cos(h), -0.02 + 0.01 * h ** 2, 1e-3 * np.sin(h), 2e-4 * h, 1e-5 * np.ones(n)])


def test_oracle_trap_table_matches_natural_spline_gradient():
    table = smooth_table()
    holder, plasma, sim, grains = fork_case(N=2, order=0, grains=[], table=table)
    lam = plasma.r_D_e
    # two ions far apart (ion–ion term exp(-100) ~ 0); the acceleration is trap + uniform field
    rng = np.random.default_rng(3)
    hs = np.linspace(-2.5, 2.5, table.shape[1])
    spl = [CubicSpline(hs, table[k], bc_type="natural") for k in range(5)]
    c = holder.cfg
    k = 1 / (4 * np.pi * c.eps_0)
    q_s = abs(c.e) * c.N_s
    m_s = c.m_i * c.N_s
    C = k * q_s * q_s / lam ** 2 / m_s  # acceleration scale of -grad_lambda P
    for _ in range(20):
        p0 = np.array([rng.uniform(-0.8, 0.8), rng.uniform(-0.8, 0.8), rng.uniform(-2.4, 2.4)])
        pos = np.array([p0, p0 + [0.0, 0.0, 100.0]]) * lam
        a = oracle.accel(holder, pos, np.zeros(0), round32=False)[0]
        u = p0[0] ** 2 + p0[1] ** 2
        dPdu = sum(kk * float(spl[kk](p0[2])) * u ** (kk - 1) for kk in range(1, 5))
        dPdh = sum(float(spl[kk](p0[2], 1)) * u ** kk for kk in range(5))
        exp = -C * np.array([2 * p0[0] * dPdu, 2 * p0[1] * dPdu, dPdh])
        exp[2] += q_s * c.E / m_s
        np.testing.assert_allclose(a, exp, rtol=1e-9, atol=1e-12 * np.abs(exp).max())


def test_oracle_field_order2_is_clamped():
    holder, plasma, sim, _ = fork_case(N=2, order=2, grains=[])
    c = holder.cfg
    q_s = abs(c.e) * c.N_s
    m_s = c.m_i * c.N_s
    lam = plasma.r_D_e
    E = lambda z: c.E + c.field_alpha * z + c.field_beta * z ** 2
    for z, zc in [(-2.4 * lam, c.field_z1), (0.3 * lam, 0.3 * lam), (2.4 * lam, c.field_z7)]:
        pos = np.array([[0.0, 0.0, z], [0.0, 0.0, z + 100 * lam]])
        a = oracle.accel(holder, pos, np.zeros(0), round32=False)
        assert a[0, 2] == pytest.approx(q_s * E(zc) / m_s, rel=1e-12)


def _kdk(holder, pos, vel, q):
    """One reference KDK without collisions (SI), from the oracle's accelerations."""
    c = holder.cfg
    a0 = oracle.accel(holder, pos, q, round32=False)
    v1 = vel + 0.5 * c.d_t * a0
    x1 = pos + c.d_t * v1
    a1 = oracle.accel(holder, x1, q, round32=False)
    return x1, v1 + 0.5 * c.d_t * a1


def test_oracle_fork_step_reflects_side_and_reinjects_top():
    lam0 = mt.PlasmaParametersInSIUnitsMatthews(290.0, 30000.0, 1e14, 0, {"E_0": [0, ""]}, 1.0, 0.0,
                                                6.6335209e-26).r_D_e
    # uncharged grains, so that an ion placed inside one stays there through the step
    grains = [mt.DustParticle(0.0, 0.0, -0.5 * lam0, 4.4e-6, "given", 0.0),
              mt.DustParticle(0.0, 0.0, 0.5 * lam0, 4.4e-6, "given", 0.0)]
    holder, plasma, sim, grains = fork_case(N=4, order=2, n=2, grains=grains)
    lam, R, H = plasma.r_D_e, sim.R, sim.H
    vT = plasma.v_T
    pos = np.array([[R * 0.999, 0.0, 0.1 * lam],          # crosses the side wall
                    [0.0, 0.0, -0.5 * lam + 1e-6],       # inside grain 0
                    [0.0, 0.3 * lam, H / 2 * 0.9999],     # leaves through the bottom plane
                    [0.2 * lam, -0.2 * lam, -1.0 * lam]])  # stays
    vel = np.array([[40 * vT, 5 * vT, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, 30 * vT], [vT, 0.0, vT]])
    q = np.array([g.q for g in grains])
    x1, v1 = _kdk(holder, pos, vel, q)
    r = oracle.run(holder, pos, vel, 0, 1, round32=False)
    # side wall: position kept, radial velocity reversed with the normal at x1
    n = np.array([x1[0, 0], x1[0, 1]]) / np.hypot(x1[0, 0], x1[0, 1])
    vn = v1[0, :2] @ n
    assert np.hypot(*x1[0, :2]) >= R
    np.testing.assert_allclose(r["pos"][0], x1[0], rtol=1e-12)
    np.testing.assert_allclose(r["vel"][0, :2], v1[0, :2] - 2 * vn * n, rtol=1e-9)
    assert r["vel"][0, 2] == pytest.approx(v1[0, 2], rel=1e-12)
    # inside a grain and past the bottom plane: re-injected on the top face z = -H/2
    for i in (1, 2):
        assert r["pos"][i, 2] == pytest.approx(-H / 2, rel=1e-12)
        assert np.hypot(*r["pos"][i, :2]) <= R
    np.testing.assert_allclose(r["pos"][3], x1[3], rtol=1e-12)
    assert r["dN"][0, 0] == 1 and r["dN"][0, 1] == 0


def test_fit_trap_table_recovers_polynomial():
    grid_R, grid_H = sh.matthews_trap_grid(1.25e-3, 5e-3, 1e-3)
    al = smooth_table(len(grid_H))
    pot = -sum(al[k][:, None] * grid_R[None, :] ** (2 * k) for k in range(5))
    np.testing.assert_allclose(sh.fit_trap_table(pot, grid_R, 4096), al, atol=1e-10)


def test_trap_file_roundtrip(tmp_path):
    al = smooth_table(50)
    f = tmp_path / "trapFile.txt"
    sh.write_trap_table(str(f), al)
    assert len(f.read_text().splitlines()) == 50
    np.testing.assert_allclose(sh.read_trap_table(str(f)), al, rtol=1e-15)


def test_out_of_domain_factor_linear_table():
    # alpha_k(h) linear in h: the quartic interpolating spline reproduces it exactly
    n, lam = 50, 1e-3
    h = np.linspace(-2.5, 2.5, n)
    al = np.vstack([0.5 + 0.1 * h, 0.02 - 0.003 * h, 1e-3 * h, 2e-4 + 0 * h, 1e-5 * h])
    eps_0, q_s = 8.85418781762039e-12, 1.6e-19 * 100
    x, y, z = 0.3e-3, -0.2e-3, 0.7e-3
    f = sh.trap_table_out_factor(al, 5e-3, lam, eps_0, q_s, [(x, y, z)])[0]
    k = 1 / (4 * np.pi * eps_0)
    r, hz = np.hypot(x, y), z / lam
    a = [al[kk][0] + (al[kk][1] - al[kk][0]) / (h[1] - h[0]) * (hz - h[0]) for kk in range(5)]
    da = [(al[kk][1] - al[kk][0]) / (h[1] - h[0]) for kk in range(5)]
    fR = sum(-2 * kk * a[kk] * r ** (2 * kk - 1) / lam ** (2 * kk) for kk in range(1, 5)) * k * q_s / lam
    fH = sum(-da[kk] * r ** (2 * kk) / lam ** (2 * kk) / lam for kk in range(5)) * k * q_s / lam
    np.testing.assert_allclose(f, [fR * x / r, fR * y / r, fH], rtol=1e-9)


def test_matthews_api_objects():
    holder, plasma, sim, grains = fork_case(N=1024, order=2)
    c = holder.cfg
    assert c.distribution == 2 and c.collision_model == 1 and c.trap_kind == 2
    assert (c.p_top, c.p_side, c.p_bottom) == (1.0, 0.0, 0.0)
    assert plasma.v_fl == pytest.approx(plasma.M * plasma.v_B)
    assert sim.r_0 == pytest.approx(1e-3 * plasma.r_D_e)
    assert c.grain_field[1] == pytest.approx(c.E + c.field_alpha * grains[1].z + c.field_beta * grains[1].z ** 2)
    from opendust.matthews import OpenDust, PlasmaParametersInSIUnitsMatthews  # noqa: F401
    od = mt.OpenDust(plasma, sim, mt.OutputParameters(trapFileName="t.txt"), grains)
    assert od.dustParticles[0].forceExternalField.shape == (sim.n, 3)
