"""Host-side setup of one simulation (FP64, numpy/scipy), computed once per simulate().

Restates the setup half of OpenDust.simulate():
  * inverse-CDF injection tables and face probabilities (opendust.py:608-837),
  * the trap fit (opendust.py:499-577), whose Monte-Carlo grid sum runs on the GPU
    (``od_trap_potential``) and whose least-squares fit runs here,
  * initial ion positions and velocities (opendust.py:370-451) and the restart-file
    reader (opendust.py:452-466).
The reference formats every table number with eight decimals in nm/ps before OpenMM
parses it (opendust.py:720-740); the tables below are rounded the same way and then
converted to SI (1 nm/ps = 1000 m/s).
"""
from __future__ import annotations

import numpy as np
from scipy import integrate, special
from scipy.interpolate import interp1d

NMPS = 1.0e3  # m/s per nm/ps


def _r8(x: float) -> float:
    return float("{:.8f}".format(x))


def _flux_maxwell(v_fl, v_T):
    def f(v):
        return v / np.sqrt(2.0 * np.pi * v_T**2) * np.exp(-((v - v_fl) ** 2) / (2.0 * v_T**2))

    return f


def _flux_field(v_fl, v_T, weight_v: bool):
    def f(v):
        base = (
            1
            / 2.0
            / abs(v_fl)
            * np.exp(-(2.0 * (v / v_T) * (v_fl / v_T) - 1) / (2.0 * (v_fl / v_T) ** 2))
            * (special.erf(((v / v_T) * (v_fl / v_T) - 1.0) / (np.sqrt(2.0) * abs((v_fl / v_T)))) + 1.0)
        )
        return v * base if weight_v else base

    return f


def _table_from_nodes(v, xi):
    """Rounded piecewise-linear inverse CDF: v[i-1] + (u - xi[i-1]) * slope[i].

    Where the CDF is flat to double precision (a tail whose flux underflows, so that two nodes
    hold the same CDF value) the interval is empty and its slope is set to 0: a draw of exactly
    that CDF value (u = 0 below a flat leading tail) then yields the node's speed instead of
    0 * inf = NaN."""
    n = len(v)
    vr = np.array([_r8(x) for x in v])
    xr = np.array([_r8(x) for x in xi])
    sl = np.zeros(n)
    for i in range(1, n):
        dx = xi[i] - xi[i - 1]
        sl[i] = _r8((v[i] - v[i - 1]) / dx) if dx > 0 else 0.0
    return vr * NMPS, xr, sl * NMPS


def v_table(v_fl: float, v_T: float, side: str, distribution: str):
    """Restates _vStringDefine (opendust.py:608-724). Speeds in nm/ps.

    Returns (F_max, (v [m/s], xi, slope [m/s])); F_max = 0 and an empty table when
    v_max < 0.4 v_T (opendust.py:631-632).
    """
    if distribution == "Maxwellian":
        if side == "top":
            v_max = v_fl + 4 * v_T
            v_min = max(v_fl - 4 * v_T, 0)
        elif side == "bottom":
            v_max = max(v_fl + 4 * v_T, 0)
            v_min = 0
        else:
            v_max = 4 * v_T
            v_min = 0
    else:
        if side == "top":
            v_max = abs(v_fl) * 6 + 5 * v_T
            v_min = 0
        else:
            v_max = 4 * v_T
            v_min = 0
    if v_max < 0.4 * v_T:
        return 0.0, (np.zeros(0), np.zeros(0), np.zeros(0))
    if distribution == "fieldDriven" and side == "top":
        n1 = int(4 * v_T / (0.2 * v_T))
        n2 = int((v_max - 5 * v_T) / v_T)
        v = np.concatenate((np.linspace(0, 4 * v_T, n1), np.linspace(5 * v_T, v_max, n2)))
    else:
        n_v = int((v_max - v_min) / (0.2 * v_T))
        v = np.linspace(v_min, v_max, n_v)
    if distribution == "Maxwellian" or side == "side":
        f = _flux_maxwell(v_fl, v_T)
    else:
        f = _flux_field(v_fl, v_T, weight_v=True)

    def F(x):
        return integrate.quad(f, v_min, x)[0]

    F_max = F(v_max)
    xi = np.array([F(x) / F_max for x in v])
    if side == "bottom":
        v = -v
    return F_max, _table_from_nodes(v, xi)


def vz_table(v_fl: float, v_T: float):
    """Restates _vZStringDefine (opendust.py:726-787): field-driven axial speed of side ions."""
    v_max = abs(v_fl) * 6 + 5 * v_T
    v_min = -4 * v_T
    n1 = int(8 * v_T / (0.2 * v_T))
    n2 = int((v_max - 5 * v_T) / v_T)
    v = np.concatenate((np.linspace(v_min, 4 * v_T, n1), np.linspace(5 * v_T, v_max, n2)))
    f = _flux_field(v_fl, v_T, weight_v=False)

    def F(x):
        return integrate.quad(f, v_min, x)[0]

    F_max = F(v_max)
    xi = np.array([F(x) / F_max for x in v])
    return _table_from_nodes(v, xi)


def injection_setup(v_fl_si: float, v_T_si: float, R_si: float, H_si: float, distribution: str):
    """Tables (top, bottom, side, vz) and face probabilities (opendust.py:789-837)."""
    v_fl = v_fl_si / NMPS
    v_T = v_T_si / NMPS
    Ft, top = v_table(v_fl, v_T, "top", distribution)
    Fb, bot = v_table(-v_fl, v_T, "bottom", distribution)
    Fs, side = v_table(0, v_T, "side", distribution)
    vz = vz_table(v_fl, v_T) if distribution == "fieldDriven" else (np.zeros(0),) * 3
    R = R_si * 1e9
    H = H_si * 1e9
    den = np.pi * R**2 * Ft + np.pi * R**2 * Fb + 2 * np.pi * R * H * Fs
    p_t = np.pi * R**2 * Ft / den
    p_s = 2 * np.pi * R * H * Fs / den
    p_b = np.pi * R**2 * Fb / den
    return [top, bot, side, vz], (p_t, p_s, p_b)


def trap_design_matrix(grid_R: np.ndarray, grid_H: np.ndarray) -> np.ndarray:
    """Columns of the 8th-degree even polynomial (opendust.py:525-546)."""
    H, R = np.meshgrid(grid_H, grid_R, copy=False)
    R = R.flatten()
    H = H.flatten()
    return np.vstack(
        [
            R * 0 + 1, R**2, H**2, H**2 * R**2, R**4, H**4, R**4 * H**2, R**2 * H**4,
            R**6, H**6, R**4 * H**4, R**6 * H**2, R**2 * H**6, R**8, H**8,
        ]
    ).T


def trap_grid(R_si: float, H_si: float, r_D_e_si: float):
    """Grid sizes and sample count of the trap fit (opendust.py:501-508)."""
    R = (R_si * 1e9) / (r_D_e_si * 1e9)
    H = (H_si * 1e9) / (r_D_e_si * 1e9)
    n_r = int(R * 10)
    n_h = int(H * 5)
    n_points = int(np.pi * R**2.0 * H / (0.05) ** 3.0)
    return R, H, n_r, n_h, n_points


def fit_trap(pot: np.ndarray, Rh: float, Hh: float, n_superions: int) -> np.ndarray:
    """Least-squares fit of the grid potential; alpha = -coef * N (opendust.py:547-550)."""
    n_r, n_h = pot.shape
    A = trap_design_matrix(np.linspace(0, Rh, n_r), np.linspace(0, Hh / 2.0, n_h))
    return -np.linalg.lstsq(A, pot.flatten(), rcond=None)[0] * n_superions


def field_driven_vz_table(v_fl: float, v_T: float):
    """Nodes (v [m/s], CDF) of the initial field-driven v_z distribution (opendust.py:405-433)."""
    v_max = abs(v_fl) * 8 + 5 * v_T
    v_min = -4 * v_T
    n_v = int((v_max - v_min) / (0.2 * v_T))
    v = np.linspace(v_min, v_max, n_v)
    f = _flux_field(v_fl, v_T, weight_v=False)
    F_max = integrate.quad(f, v_min, v_max)[0]
    xi = np.array([integrate.quad(f, v_min, x)[0] / F_max for x in v])
    return v, xi


def field_driven_vz(v_fl: float, v_T: float, u: np.ndarray) -> np.ndarray:
    """Initial field-driven v_z by inverse CDF (opendust.py:405-448); speeds in m/s."""
    v, xi = field_driven_vz_table(v_fl, v_T)
    return interp1d(xi, v)(u)


def initial_state(N: int, R: float, H: float, grains: list, v_fl: float, v_T: float,
                  distribution: str, seed: int):
    """Uniform positions in the cylinder outside every grain, drifting Maxwellian (or
    field-driven) velocities; SI units. Restates opendust.py:373-451, vectorised, with a
    seeded numpy generator in place of the reference's global RNG."""
    rng = np.random.default_rng(seed)
    pos = np.empty((0, 3))
    while pos.shape[0] < N:
        m = int((N - pos.shape[0]) * 1.1) + 16
        r = np.sqrt(rng.uniform(0, 1, m))
        th = rng.uniform(0, 1, m)
        x = R * r * np.cos(2 * np.pi * th)
        y = R * r * np.sin(2 * np.pi * th)
        z = rng.uniform(-H / 2, H / 2, m)
        ok = np.ones(m, dtype=bool)
        for g in grains:
            d = np.sqrt((x - g[0]) ** 2 + (y - g[1]) ** 2 + (z - g[2]) ** 2)
            ok &= d > g[3]
        pos = np.concatenate([pos, np.stack([x, y, z], 1)[ok]])
    pos = pos[:N]
    vel = np.empty((N, 3))
    vel[:, 0] = rng.normal(0, v_T, N)
    vel[:, 1] = rng.normal(0, v_T, N)
    if distribution == "Maxwellian":
        vel[:, 2] = rng.normal(v_fl, v_T, N)
    else:
        vel[:, 2] = field_driven_vz(v_fl, v_T, rng.uniform(0, 1, N))
    return pos, vel


def read_restart(path: str, N: int):
    """Restart file: one ion per line, ``x y z vx vy vz`` tab-separated in nm and nm/ps
    (opendust.py:452-466, :1100-1115). Returns SI arrays."""
    from . import _lib
    try:
        p, v = _lib.read_restart_file(path, N)
    except _lib.OpenDustError as e:
        raise ValueError(str(e)) from None
    return p * 1e-9, v * NMPS


def write_restart(path: str, pos: np.ndarray, vel: np.ndarray):
    """Same format as read_restart, the reference's bytes (numbers as Python's "{}".format)."""
    from . import _lib
    _lib.write_restart_file(path, np.asarray(pos) * 1e9, np.asarray(vel) / NMPS)


# ----------------------------------------------------------------- chains/matthews.py fork
def matthews_trap_grid(R: float, H: float, r_D_e: float):
    """Grid of the fork's trap fit in units of r_D_e (chains/matthews.py:398-405): int(10 R)
    radii on [0, R] and int(10 H) heights on [-H/2, H/2]."""
    Rh, Hh = R / r_D_e, H / r_D_e
    return np.linspace(0.0, Rh, int(Rh * 10)), np.linspace(-Hh / 2.0, Hh / 2.0, int(Hh * 10))


def fit_trap_table(pot: np.ndarray, grid_R: np.ndarray, N: int) -> np.ndarray:
    """Per-height least squares of the fork (chains/matthews.py:420-440): pot[j, i] is the
    summed screened potential of the N ions at (grid_R[i], 0, h_j); returns alpha (5, n_h),
    alpha[k, j] the coefficient of rho^(2k) at height h_j (rho in units of r_D_e)."""
    potential = np.asarray(pot, dtype=np.float64) / float(N)
    A = np.vstack([np.ones(len(grid_R)), grid_R ** 2, grid_R ** 4, grid_R ** 6, grid_R ** 8]).T
    alpha = np.zeros((5, potential.shape[0]))
    for j in range(potential.shape[0]):
        alpha[:, j] = -np.linalg.lstsq(A, potential[j], rcond=None)[0] * N
    return alpha


def read_trap_table(path: str) -> np.ndarray:
    """Trap file of the fork (chains/matthews.py:441-453): one height per line, the five
    coefficients tab-separated. Returns (5, n)."""
    return np.loadtxt(path, delimiter="\t", ndmin=2)[:, :5].T.copy()


def write_trap_table(path: str, alpha: np.ndarray):
    """Same format (chains/matthews.py:827-833)."""
    with open(path, "w") as f:
        for j in range(alpha.shape[1]):
            f.write("{}\t{}\t{}\t{}\t{}\n".format(*(alpha[k][j] for k in range(5))))


def trap_table_out_factor(alpha: np.ndarray, H: float, r_D_e: float, eps_0: float, q_s: float,
                          grains_xyz) -> np.ndarray:
    """Out-of-domain trap force on each grain per unit grain charge [N/C] for the tabulated
    trap (chains/matthews.py:975-1013): quartic interpolating splines of the alpha_k(h) rows
    (scipy UnivariateSpline k=4, s=0, as the fork) and their derivatives at the grain height.
    Returns (P, 3)."""
    from scipy.interpolate import UnivariateSpline

    hs = np.linspace(-H / r_D_e / 2.0, H / r_D_e / 2.0, alpha.shape[1])
    spl = [UnivariateSpline(hs, alpha[k], k=4, s=0) for k in range(5)]
    der = [s.derivative() for s in spl]
    k = 1.0 / (eps_0 * 4.0 * np.pi)
    L = r_D_e
    out = np.zeros((len(grains_xyz), 3))
    for p, (x, y, z) in enumerate(grains_xyz):
        r = np.sqrt(x ** 2 + y ** 2)
        h = z / L
        fR = (-2 * float(spl[1](h)) * r) / L ** 2
        fR += (-4 * float(spl[2](h)) * r ** 3) / L ** 4
        fR += (-6 * float(spl[3](h)) * r ** 5) / L ** 6
        fR += (-8 * float(spl[4](h)) * r ** 7) / L ** 8
        fR *= k * q_s / L
        fH = (-float(der[0](h))) / L
        fH += (-float(der[1](h)) * r ** 2) / L ** 2 / L
        fH += (-float(der[2](h)) * r ** 4) / L ** 4 / L
        fH += (-float(der[3](h)) * r ** 6) / L ** 6 / L
        fH += (-float(der[4](h)) * r ** 8) / L ** 8 / L
        fH *= k * q_s / L
        out[p] = (0.0, 0.0, fH) if r == 0 else (fR * x / r, fR * y / r, fH)
    return out


def matthews_field_at(order: int, Phi: dict, z: float) -> float:
    """Field along z at a grain [V/m] as the fork's tail uses it (chains/matthews.py:1086-1095):
    E_0 for order 0, E_0 + alpha z + beta z^2 (not clamped) for order 2."""
    E0 = Phi["E_0"][0]
    if order == 2:
        return E0 + Phi["alpha"][0] * z + Phi["beta"][0] * z ** 2
    return E0
