"""Seeded synthetic particle sets with the shapes of the benchmark workloads.

Each generator returns a dict of float64 numpy arrays in SoA form
(``x y z vx vy vz m u h``) plus the run parameters the workload uses.  The smoothing
length ``h`` is an analytic first guess h = h_fac (m / rho_model)^(1/3); the h-rho
solve refines it.  None of these reuse the reference's IC generators; where a shape
mirrors one (Plummer velocities, src/Ic/PlummerSphereIc.cpp:134-146), the method is the
published Aarseth, Henon & Wielen (1974) rejection sampler.
"""
from __future__ import annotations

import math

import numpy as np

H_FAC = 1.2


def _pack(x, v, m, u, h):
    return {
        "x": np.ascontiguousarray(x[:, 0]), "y": np.ascontiguousarray(x[:, 1]),
        "z": np.ascontiguousarray(x[:, 2]),
        "vx": np.ascontiguousarray(v[:, 0]), "vy": np.ascontiguousarray(v[:, 1]),
        "vz": np.ascontiguousarray(v[:, 2]),
        "m": np.ascontiguousarray(m), "u": np.ascontiguousarray(u),
        "h": np.ascontiguousarray(h),
    }


def periodic_cube(n: int = 32768, seed: int = 1234) -> dict:
    """Uniform random particles in the periodic unit cube [0,1)^3 (hydro only).

    Equal masses summing to 1, u = 1 +- 1 % uniform noise, Gaussian velocities with
    sigma = 0.1 per axis, gamma = 5/3.
    """
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3))
    v = rng.normal(0.0, 0.1, (n, 3))
    m = np.full(n, 1.0 / n)
    u = 1.0 + 0.01 * (2.0 * rng.random(n) - 1.0)
    h = np.full(n, H_FAC * (1.0 / n) ** (1.0 / 3.0))
    ics = _pack(x, v, m, u, h)
    ics["params"] = dict(self_gravity=0, eos=0, periodic=1, boxmin=(0.0, 0.0, 0.0),
                         boxmax=(1.0, 1.0, 1.0), gamma_eos=5.0 / 3.0, thetamaxsqd=0.25)
    return ics


def plummer_sphere(n: int = 262144, seed: int = 4321, rtrunc: float = 10.0) -> dict:
    """Plummer sphere (a = M = G = 1) of gas, truncated at ``rtrunc`` scale radii.

    Radii are drawn from the cumulative mass M(<r) = r^3 / (1 + r^2)^(3/2); speeds from
    the isotropic distribution function by rejection on g(q) = q^2 (1 - q^2)^(7/2),
    v = q v_esc(r), v_esc = sqrt(2) (1 + r^2)^(-1/4).  u = 0.05.
    """
    rng = np.random.default_rng(seed)
    mtrunc = rtrunc ** 3 / (1.0 + rtrunc ** 2) ** 1.5
    xm = rng.random(n) * mtrunc
    xm = np.maximum(xm, 1e-300)
    r = 1.0 / np.sqrt(xm ** (-2.0 / 3.0) - 1.0)
    x = r[:, None] * _unit_vectors(rng, n)
    q = np.empty(n)
    todo = np.arange(n)
    while todo.size:
        qq = rng.random(todo.size)
        yy = 0.1 * rng.random(todo.size)
        ok = yy < qq * qq * (1.0 - qq * qq) ** 3.5
        q[todo[ok]] = qq[ok]
        todo = todo[~ok]
    vesc = math.sqrt(2.0) * (1.0 + r * r) ** -0.25
    v = (q * vesc)[:, None] * _unit_vectors(rng, n)
    m = np.full(n, 1.0 / n)
    u = np.full(n, 0.05)
    rho = 3.0 / (4.0 * math.pi) * (1.0 + r * r) ** -2.5
    h = H_FAC * (m / rho) ** (1.0 / 3.0)
    ics = _pack(x, v, m, u, h)
    ics["params"] = dict(self_gravity=1, eos=0, periodic=0, thetamaxsqd=0.25, gamma_eos=5.0 / 3.0)
    return ics


def evrard_sphere(n: int = 8388608, seed: int = 51, nstar: int = 64) -> dict:
    """Evrard collapse initial state: gas sphere R = M = G = 1 with rho ~ 1/r (r = R sqrt(U),
    isotropic directions), u = 0.05 G M / R, at rest; plus ``nstar`` stars of mass 1e-3,
    uniform in r < 0.5, at rest, softening length h = 0.01 (with_stars)."""
    rng = np.random.default_rng(seed)
    r = np.sqrt(rng.random(n))
    x = r[:, None] * _unit_vectors(rng, n)
    v = np.zeros((n, 3))
    m = np.full(n, 1.0 / n)
    u = np.full(n, 0.05)
    rho = 1.0 / (2.0 * math.pi * np.maximum(r, 1e-6))
    h = H_FAC * (m / rho) ** (1.0 / 3.0)
    ics = _pack(x, v, m, u, h)
    ics["params"] = dict(self_gravity=1, eos=0, periodic=0, thetamaxsqd=0.25, gamma_eos=5.0 / 3.0)
    if nstar:
        ics = with_stars(ics, nstar, rmax=0.5, mass=1.0e-3, h=0.01, seed=seed + 1)
    return ics


def rotating_cloud(n: int = 1048576, seed: int = 31, amp: float = 0.1, erot: float = 0.16,
                   etherm: float = 0.26) -> dict:
    """Uniform rotating sphere (R = M = G = 1) with an m = 2 density perturbation.

    rho ~ 1 + amp cos(2 phi), imposed by displacing the azimuth of a uniform sphere:
    phi + (amp/2) sin(2 phi) = phi_uniform, solved by Newton iteration.  Solid-body rotation
    about z with E_rot / |E_grav| = erot (E_grav = -3/5, I = 2/5: omega^2 = erot 0.6 / 0.2);
    isothermal gas with E_therm / |E_grav| = etherm, E_therm = (3/2) M c_s^2, c_s^2 = temp0 /
    mu_bar (mu_bar = 1).
    """
    rng = np.random.default_rng(seed)
    r = rng.random(n) ** (1.0 / 3.0)
    cost = 2.0 * rng.random(n) - 1.0
    phi0 = 2.0 * math.pi * rng.random(n)
    phi = phi0.copy()
    for _ in range(30):
        f = phi + 0.5 * amp * np.sin(2.0 * phi) - phi0
        phi -= f / (1.0 + amp * np.cos(2.0 * phi))
    sint = np.sqrt(1.0 - cost * cost)
    x = np.stack([r * sint * np.cos(phi), r * sint * np.sin(phi), r * cost], 1)
    omega = math.sqrt(erot * 0.6 / 0.2)
    v = np.stack([-omega * x[:, 1], omega * x[:, 0], np.zeros(n)], 1)
    m = np.full(n, 1.0 / n)
    cs2 = etherm * 0.6 / 1.5
    gamma = 5.0 / 3.0
    u = np.full(n, cs2 / (gamma - 1.0))
    rho = 3.0 / (4.0 * math.pi) * (1.0 + amp * np.cos(2.0 * phi))
    h = H_FAC * (m / rho) ** (1.0 / 3.0)
    ics = _pack(x, v, m, u, h)
    ics["params"] = dict(self_gravity=1, eos=1, periodic=0, thetamaxsqd=0.25, gamma_eos=gamma,
                         temp0=cs2, mu_bar=1.0)
    ics["kdk"] = dict(nlevels=4, level_diff_max=1, courant_mult=0.15, accel_mult=0.3, energy_mult=0.4)
    return ics


def kh_box(n: int = 32768, seed: int = 7, pressure: float = 2.5) -> dict:
    """Periodic 3-D Kelvin-Helmholtz box [0,1) x [0,1) x [0,0.25) (hydro only).

    Equal-mass particles, density 2 in the band |y - 0.5| < 0.25 and 1 outside (2:1 in
    number density, uniform random positions in each region); shear vx = -0.5 inside and
    +0.5 outside the band; vy = 0.01 sin(4 pi x); uniform pressure P (u = P / ((gamma-1)
    rho)); gamma = 5/3.
    """
    rng = np.random.default_rng(seed)
    gamma = 5.0 / 3.0
    nd = int(round(2.0 * n / 3.0))
    nl = n - nd
    xd = np.stack([rng.random(nd), 0.25 + 0.5 * rng.random(nd), 0.25 * rng.random(nd)], 1)
    yl = 0.5 * rng.random(nl)
    yl = np.where(yl < 0.25, yl, yl + 0.5)
    xl = np.stack([rng.random(nl), yl, 0.25 * rng.random(nl)], 1)
    x = np.concatenate([xd, xl])
    dense = np.concatenate([np.ones(nd, bool), np.zeros(nl, bool)])
    rho = np.where(dense, 2.0, 1.0)
    v = np.zeros((n, 3))
    v[:, 0] = np.where(dense, -0.5, 0.5)
    v[:, 1] = 0.01 * np.sin(4.0 * math.pi * x[:, 0])
    mtot = 2.0 * 0.5 * 0.25 + 1.0 * 0.5 * 0.25
    m = np.full(n, mtot / n)
    u = pressure / ((gamma - 1.0) * rho)
    h = H_FAC * (m / rho) ** (1.0 / 3.0)
    ics = _pack(x, v, m, u, h)
    ics["params"] = dict(self_gravity=0, eos=0, periodic=1, boxmin=(0.0, 0.0, 0.0),
                         boxmax=(1.0, 1.0, 0.25), gamma_eos=gamma, thetamaxsqd=0.25)
    return ics


def kh_ensemble(nbox: int = 64, nmin: int = 4096, nmax: int = 131072, seed: int = 2024) -> list:
    """``nbox`` independent KH boxes with particle counts log-uniform in [nmin, nmax]."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(math.log(nmin), math.log(nmax), nbox)).astype(int)
    return [kh_box(int(nb), seed=seed + 1 + i) for i, nb in enumerate(sizes)]


def with_stars(ics: dict, nstar: int = 64, rmax: float = 0.5, mass: float = 1.0e-3, h: float = 0.01,
               sigma_v: float = 0.0, seed: int = 99) -> dict:
    """Add ``nstar`` star particles, uniform in the sphere r < rmax, to a particle set.

    Stars carry x y z vx vy vz m h (h: the star's softening length, used in the mean-h
    kernel of the SPH-star gravity); velocities are Gaussian with ``sigma_v`` per axis.
    """
    rng = np.random.default_rng(seed)
    r = rmax * rng.random(nstar) ** (1.0 / 3.0)
    x = r[:, None] * _unit_vectors(rng, nstar)
    v = rng.normal(0.0, sigma_v, (nstar, 3)) if sigma_v > 0 else np.zeros((nstar, 3))
    ics = dict(ics)
    ics["stars"] = {"x": x[:, 0].copy(), "y": x[:, 1].copy(), "z": x[:, 2].copy(),
                    "vx": v[:, 0].copy(), "vy": v[:, 1].copy(), "vz": v[:, 2].copy(),
                    "m": np.full(nstar, mass), "h": np.full(nstar, h)}
    return ics


def _unit_vectors(rng, n):
    cost = 2.0 * rng.random(n) - 1.0
    phi = 2.0 * math.pi * rng.random(n)
    sint = np.sqrt(1.0 - cost * cost)
    return np.stack([sint * np.cos(phi), sint * np.sin(phi), cost], axis=1)


WORKLOADS = {
    "periodic_cube": periodic_cube,
    "plummer_sphere": plummer_sphere,
    "kh_box": kh_box,
    "rotating_cloud": rotating_cloud,
    "evrard_sphere": evrard_sphere,
}
