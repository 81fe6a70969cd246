"""CPU tests pinning the oracle: published Philox vectors and analytic known answers."""
import math

import numpy as np
import pytest
from scipy import integrate, stats

from opendust_gb300 import build_simulation, setup_host, workloads
from oracle import oracle

ZERO_TRAP = np.zeros(15)


def _cfg(N=2, builder=workloads.small_plain, trap=ZERO_TRAP, **kw):
    plasma, sim, grains, dist, ext = builder(N=N, n=4)
    holder, info = build_simulation(plasma, sim, grains, dist, trap=trap, **{**ext, **kw})
    return holder, plasma, sim, grains


# Random123 known-answer vectors for Philox4x32-10
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,out", KAT)
def test_philox_kat(ctr, key, out):
    assert oracle.philox(ctr, key) == out


def yukawa_force(plasma, sim, xi, xj):
    """Force on i from j of U = k q_s^2 exp(-r/lambda)/(r + r_0) (opendust.py:472)."""
    k = 1 / (4 * np.pi * plasma.eps_0)
    q_s = abs(plasma.e) * sim.N_s
    lam, r0 = plasma.r_D_e, sim.r_0
    d = np.asarray(xi) - np.asarray(xj)
    r = np.linalg.norm(d)
    s = r + r0
    mag = k * q_s**2 * np.exp(-r / lam) * (1 / (lam * s) + 1 / s**2)
    return mag * d / r


def test_two_ion_yukawa():
    holder, plasma, sim, _ = _cfg(N=2)
    lam = plasma.r_D_e
    for d in (1e-3, 0.01, 0.3, 1.0, 2.5):
        pos = np.array([[0.1 * lam, 0.2 * lam, -0.3 * lam], [0.1 * lam + d * lam, 0.2 * lam, -0.3 * lam]])
        f = oracle.force_snapshot(holder, pos, round32=False)
        ref = yukawa_force(plasma, sim, pos[0], pos[1])
        np.testing.assert_allclose(f[0], ref, rtol=1e-12, atol=1e-30)
        np.testing.assert_allclose(f[1], -ref, rtol=1e-12, atol=1e-30)


def test_three_ion_superposition():
    holder, plasma, sim, _ = _cfg(N=3)
    lam = plasma.r_D_e
    pos = np.array([[0, 0, 0], [0.4, 0.1, 0.0], [-0.2, 0.5, 0.3]]) * lam
    f = oracle.force_snapshot(holder, pos, round32=False)
    for i in range(3):
        ref = sum(yukawa_force(plasma, sim, pos[i], pos[j]) for j in range(3) if j != i)
        np.testing.assert_allclose(f[i], ref, rtol=1e-12)


def test_ion_grain_coulomb_and_field():
    holder, plasma, sim, grains = _cfg(N=2)
    lam = plasma.r_D_e
    q = np.array([-2.5e-15])
    pos = np.array([[0.05 * lam, -0.02 * lam, 0.03 * lam], [500 * lam, 0, 0]])
    a = oracle.accel(holder, pos, q, round32=False)
    k = 1 / (4 * np.pi * plasma.eps_0)
    q_s = abs(plasma.e) * sim.N_s
    m_s = plasma.m_i * sim.N_s
    d = pos[0]
    ref = k * q[0] * q_s * d / np.linalg.norm(d) ** 3 / m_s
    np.testing.assert_allclose(a[0], ref, rtol=1e-12)
    # field-driven: F_z = E q_s added on every ion (opendust.py:580-585)
    holder2, plasma2, sim2, _ = _cfg(N=2, builder=workloads.field_chain, collisions="none",
                                     cutoff_distance=None)
    pos2 = np.array([[0.0, 2.5 * plasma2.r_D_e, 0.0], [0.0, -2.5 * plasma2.r_D_e, 400 * plasma2.r_D_e]])
    a2 = oracle.accel(holder2, pos2, np.zeros(5), round32=False)
    q_s2 = abs(plasma2.e) * sim2.N_s
    m_s2 = plasma2.m_i * sim2.N_s
    assert a2[1, 2] == pytest.approx(plasma2.E * q_s2 / m_s2, rel=1e-9)


def test_trap_gradient():
    alpha = np.linspace(0.3, -0.2, 15) * 10
    holder, plasma, sim, _ = _cfg(N=2, trap=alpha)
    lam = plasma.r_D_e
    k = 1 / (4 * np.pi * plasma.eps_0)
    q_s = abs(plasma.e) * sim.N_s
    m_s = plasma.m_i * sim.N_s
    A = setup_host.trap_design_matrix

    def U(x):  # energy of opendust.py:552-577 in J
        r = math.hypot(x[0], x[1]) / lam
        h = x[2] / lam
        cols = A(np.array([r]), np.array([h]))[0]
        return k * q_s**2 / lam * float(np.dot(alpha[1:], cols[1:]))

    x0 = np.array([0.7, -1.1, 1.3]) * lam
    pos = np.array([x0, [900 * lam, 0, 0]])
    a = oracle.accel(holder, pos, np.zeros(1), round32=False)[0]
    eps = 1e-6 * lam
    grad = np.array([(U(x0 + eps * e) - U(x0 - eps * e)) / (2 * eps) for e in np.eye(3)])
    np.testing.assert_allclose(a, -grad / m_s, rtol=1e-6)


def test_flags_on_surfaces_inclusive():
    holder, plasma, sim, grains = _cfg(N=8)
    g = grains[0]
    pos = np.array([
        [g.r, 0, 0],                 # on the grain surface: inside (step(0) = 1)
        [0, 0, 0.5 * g.r],           # inside
        [sim.R, 0, 0],               # on the side wall: outside_domain_r
        [0, 0, sim.H / 2],           # on the top/bottom planes: outside_domain_z
        [0, 0, -sim.H / 2],
        [0.5 * sim.R, 0.5 * sim.R, 0.0],  # interior
        [0, 0, 2 * g.r],             # outside the grain
        [np.nextafter(sim.R, 0), 0, 0],
    ])
    idx, cnt, gc = oracle.collect_flags(holder, pos, round32=False)
    assert list(idx) == [0, 1, 2, 3, 4]
    assert cnt == 5 and list(gc) == [2]


def test_charge_update_closed_forms():
    for method in ("consistent", "oml"):
        plasma, sim, grains, dist, ext = workloads.small_plain(N=2, n=3)
        grains[0].chargeCalculationMethod = method
        grains[0].q = -1e-15
        holder, _ = build_simulation(plasma, sim, grains, dist, trap=ZERO_TRAP)
        lam = plasma.r_D_e
        pos = np.array([[1.0 * lam, 0, 0], [-1.0 * lam, 0, 0]])
        vel = np.zeros((2, 3))
        r = oracle.run(holder, pos, vel, 0, 3, round32=False)
        k = 1 / (4 * np.pi * plasma.eps_0)
        q = -1e-15
        rg = grains[0].r
        S = 4 * np.pi * rg**2
        expect = [q]
        for _ in range(2):
            phi = k * q / rg
            ge = plasma.n_inf * np.sqrt(plasma.T_e * plasma.k_B / np.pi / plasma.m_e / 2) * np.exp(
                -plasma.e * phi / plasma.T_e / plasma.k_B)
            if method == "consistent":
                q = q + ge * sim.d_t * S * plasma.e
            else:
                u = plasma.v_fl / plasma.v_T / np.sqrt(2)
                chi = plasma.e * phi / plasma.T_n / plasma.k_B
                gi = plasma.n_inf * plasma.v_T * np.sqrt(2) * u / 4 * (
                    (1 + 1 / (4 * u) + chi / u**2) * math.erf(u) + 1 / u / np.sqrt(np.pi) * np.exp(-u * u))
                q = q + gi * sim.d_t * S * abs(plasma.e) + ge * sim.d_t * S * plasma.e
            expect.append(q)
        np.testing.assert_allclose(r["q"][:, 0], expect, rtol=1e-12)


def test_trap_potential_matches_independent_mc():
    Rh, Hh, n_r, n_h, _ = setup_host.trap_grid(3.0, 6.0, 1.0)
    pot = oracle.trap_potential(Rh, Hh, 4, 3, 400_000, 5)
    rng = np.random.default_rng(0)
    n = 400_000
    r = np.sqrt(rng.uniform(0, 1, n)) * Rh
    th = rng.uniform(0, 2 * np.pi, n)
    x, y, z = r * np.cos(th), r * np.sin(th), rng.uniform(-Hh / 2, Hh / 2, n)
    for i, gr in enumerate(np.linspace(0, Rh, 4)):
        for j, gh in enumerate(np.linspace(0, Hh / 2, 3)):
            d = np.sqrt((gr - x) ** 2 + y**2 + (gh - z) ** 2)
            v = np.exp(-d) / (d + 0.001)
            assert abs(pot[i, j] - v.mean()) < 5 * v.std() / np.sqrt(n)


def test_injection_statistics():
    holder, plasma, sim, _ = _cfg(N=2)
    n = 20000
    faces = np.zeros(3)
    vz_top = []
    for i in range(n):
        x, v = oracle.inject(holder, i, 7)
        if x[2] <= -sim.H / 2 * (1 - 1e-12):
            faces[0] += 1
            vz_top.append(v[2])
        elif x[2] >= sim.H / 2 * (1 - 1e-12):
            faces[2] += 1
        else:
            faces[1] += 1
            assert abs(math.hypot(x[0], x[1]) - sim.R) < 1e-9 * sim.R
            assert v[0] * x[0] + v[1] * x[1] <= 0  # side ions move inward
    p = np.array([holder.cfg.p_top, holder.cfg.p_side, holder.cfg.p_bottom])
    assert np.all(np.abs(faces / n - p) < 5 * np.sqrt(p * (1 - p) / n) + 1e-12)
    # top-face v_z follows the flux-weighted shifted Maxwellian truncated to the table range
    v_fl, v_T = plasma.v_fl, plasma.v_T
    lo, hi = max(v_fl - 4 * v_T, 0), v_fl + 4 * v_T
    f = lambda v: v * np.exp(-((v - v_fl) ** 2) / (2 * v_T**2))
    Z = integrate.quad(f, lo, hi)[0]
    cdf = np.vectorize(lambda v: integrate.quad(f, lo, min(max(v, lo), hi))[0] / Z)
    ks = stats.kstest(np.array(vz_top), cdf)
    assert ks.pvalue > 1e-3


def test_injection_tables_shape():
    plasma, sim, grains, dist, _ = workloads.small_plain(N=2, n=2)
    tables, probs = setup_host.injection_setup(plasma.v_fl, plasma.v_T, sim.R, sim.H, dist)
    assert abs(sum(probs) - 1) < 1e-12
    for t in (0, 2):
        v, xi, sl = tables[t]
        assert xi[0] == 0.0 and xi[-1] == 1.0
        assert np.all(np.diff(xi) >= 0)
    assert len(tables[1][0]) == 0 and probs[2] == 0.0  # M = 1: no bottom injection
    # field-driven adds the side v_z table
    p2, s2, g2, d2, _ = workloads.field_chain(N=2, n=2)
    t2, pr2 = setup_host.injection_setup(p2.v_fl, p2.v_T, s2.R, s2.H, d2)
    assert len(t2[3][0]) > 10 and abs(sum(pr2) - 1) < 1e-12


def test_two_ion_cutoff_switching():
    # OpenMM's switching function on the energy (opendust.py:481-485): U(r) S(x), S = 1 - 10x^3
    # + 15x^4 - 6x^5, x = (r - r_s)/(r_c - r_s) on [r_s, r_c]; S = 1 below r_s, the force 0 above
    # r_c. The reference force is the central difference of the switched energy.
    holder, plasma, sim, _ = _cfg(N=2, builder=workloads.field_chain)
    c = holder.cfg
    lam = plasma.r_D_e
    rc, rs = c.cutoff, c.switch_dist
    assert rc == pytest.approx(2 * lam) and rs == pytest.approx(2 * lam * 3.0 / 3.2)
    k = 1 / (4 * np.pi * plasma.eps_0)
    q_s = abs(plasma.e) * sim.N_s

    def energy(r):
        x = min(max((r - rs) / (rc - rs), 0.0), 1.0)
        return k * q_s**2 * math.exp(-r / lam) / (r + sim.r_0) * (1 - 10 * x**3 + 15 * x**4 - 6 * x**5)

    for d in (0.5, 1.8, 1.88, 1.93, 1.99, 2.01, 2.5):
        r = d * lam
        pos = np.array([[0.2 * lam, -0.1 * lam, 0.3 * lam], [0.2 * lam + r, -0.1 * lam, 0.3 * lam]])
        f = oracle.force_snapshot(holder, pos, round32=False)
        h = 1e-7 * lam
        mag = -(energy(r + h) - energy(r - h)) / (2 * h)  # force along +d on ion 1, -d on ion 0
        np.testing.assert_allclose(f[1, 0], mag, rtol=1e-6, atol=1e-12 * abs(mag) + 1e-300)
        np.testing.assert_allclose(f[0, 0], -mag, rtol=1e-6, atol=1e-12 * abs(mag) + 1e-300)
        if d > 2.0:
            assert f[1, 0] == 0.0


def test_mfp_collisions_of_ions_faster_than_the_majorant():
    # constant mean free path (null collision with the majorant vmax = 3|v_fl| + 10 v_T): an ion
    # faster than vmax collides with its own probability 1 - exp(-|v| d_t / mfp), not the
    # majorant's. Ions at 2 vmax, mfp chosen so that vmax d_t / mfp = 0.5: 1 - e^-1 = 0.632
    # collide in one step (a capped rate would give 1 - e^-0.5 = 0.393).
    plasma0, sim0, *_ = workloads.small_plain(N=2, n=4)
    vmax = 3 * abs(plasma0.v_fl) + 10 * plasma0.v_T
    mfp = 2 * vmax * sim0.d_t
    N = 4000
    holder, plasma, sim, grains = _cfg(N=N, collisions="mfp", mean_free_path=mfp)
    rng = np.random.default_rng(4)
    lam = plasma.r_D_e
    r = 2.5 * lam * np.sqrt(rng.uniform(0, 1, N))
    th = rng.uniform(0, 2 * np.pi, N)
    pos = np.stack([r * np.cos(th), r * np.sin(th), rng.uniform(-2.5, -1.5, N) * lam], 1)
    d = rng.normal(size=(N, 3))
    vel = 2 * vmax * d / np.linalg.norm(d, axis=1, keepdims=True)
    out = oracle.run(holder, pos, vel, 0, 1, round32=False)
    collided = np.linalg.norm(out["vel"], axis=1) < vmax
    p = collided.mean()
    expect = 1 - math.exp(-1.0)
    assert abs(p - expect) < 4 * math.sqrt(expect * (1 - expect) / N), (p, expect)


def test_cutoff_cell_list_equals_double_loop():
    # Above 4096 ions the oracle's cutoff force walks a cell list; at or below it, a plain double
    # loop. Only neighbours within r_c contribute, so the force on a target from all 8000 ions
    # (cell list) must equal the force from the subset within r_c + 0.01 lambda (double loop).
    holder, plasma, sim, grains = _cfg(N=8000, builder=workloads.field_chain)
    lam = plasma.r_D_e
    pos, _ = setup_host.initial_state(8000, sim.R, sim.H, [(g.x, g.y, g.z, g.r) for g in grains],
                                      plasma.v_fl, plasma.v_T, "fieldDriven", 5)
    rc = holder.cfg.cutoff
    for t in (17, 4711):
        near = np.flatnonzero(np.linalg.norm(pos - pos[t], axis=1) < rc + 0.01 * lam)
        assert 100 < len(near) <= 4096
        f_all = oracle.force_targets(holder, pos, [t], round32=False)[0]
        sub = pos[near]
        f_sub = oracle.force_targets(holder, sub, [int(np.flatnonzero(near == t)[0])], round32=False)[0]
        np.testing.assert_allclose(f_all, f_sub, rtol=1e-11, atol=1e-12 * np.linalg.norm(f_sub))


def test_device_state_rounding():
    # oracle.DEVICE_STATE starts a run from the device's cell-relative position state: per axis a
    # cell of side s (the smallest power of two not below max(R, H/2) / 256, in lambda) and the
    # offset rounded once to float, so every coordinate is within 2^-25 s of the input; plain
    # float rounding (round32=True) is only within half an ulp of |x|
    from tests._util import case

    holder, pos, vel, plasma, sim, grains = case(N=512, n=2, seed=3, trap=np.zeros(15))
    lam = plasma.r_D_e
    s = 2.0 ** np.ceil(np.log2(max(sim.R, sim.H / 2) / lam / 256))
    rel = oracle.run(holder, pos, vel, 0, 0, round32=oracle.DEVICE_STATE)["pos"]
    f32 = oracle.run(holder, pos, vel, 0, 0, round32=True)["pos"]
    d_rel = np.max(np.abs(rel - pos)) / lam
    d_f32 = np.max(np.abs(f32 - pos)) / lam
    assert d_rel <= s * 2.0**-25 * (1 + 1e-9)
    assert d_f32 > 50 * d_rel
