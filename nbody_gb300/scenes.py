"""Seeded synthetic scenes in the reference's Body layout.

Every generator returns ``float32`` bodies of shape ``(n, 12)`` -- pos xyz, radius, vel
xyz, mass, acc xyz, pad (include/nbody/body.h:6-19) -- from numpy's counter-based Philox
generator, so a seed names one input exactly. None of these distributions is in the
reference (its own generators are util::disk and util::cube, source/util.cpp:14-126);
they are the workloads the solver is measured on:

* :func:`plummer` -- Plummer sphere sampled as Aarseth, Henon & Wielen (1974), in units
  G = M = a = 1 (then scaled), centre-of-mass frame, truncated at ``rmax``.
* :func:`two_plummer` -- two such spheres on a grazing approach.
* :func:`uniform_cube` -- uniform positions in [0,1)^3, log-normal masses summing to 1.
* :func:`batch_plummer` -- many Plummer systems with log-uniform sizes.
* :func:`disk_halo` -- exponential disk inside a Hernquist (1990) halo.
"""
from __future__ import annotations

import numpy as np


def rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(seed))


def _bodies(pos, vel, mass, radius=0.0) -> np.ndarray:
    n = len(mass)
    b = np.zeros((n, 12), np.float32)
    b[:, 0:3] = pos
    b[:, 3] = radius
    b[:, 4:7] = vel
    b[:, 7] = mass
    return b


def _isotropic(g: np.random.Generator, n: int) -> np.ndarray:
    """Unit vectors uniform on the sphere."""
    z = g.uniform(-1.0, 1.0, n)
    phi = g.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    return np.stack([s * np.cos(phi), s * np.sin(phi), z], axis=1)


def plummer_f64(n: int, seed: int, a: float = 1.0, mass: float = 1.0, G: float = 1.0,
                rmax: float = 20.0) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Plummer sphere in double precision: (pos, vel, mass) in the centre-of-mass frame.

    Radii from the inverted cumulative mass, r = a / sqrt(X^(-2/3) - 1), redrawn beyond
    rmax*a; speeds q*v_esc with q drawn from q^2 (1-q^2)^(7/2) by rejection, directions
    isotropic. Velocities scale as sqrt(G*M/a)."""
    g = rng(seed)
    r = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        x = g.uniform(1e-12, 1.0, len(todo))
        rr = 1.0 / np.sqrt(x ** (-2.0 / 3.0) - 1.0)
        ok = rr <= rmax
        r[todo[ok]] = rr[ok]
        todo = todo[~ok]
    pos = _isotropic(g, n) * r[:, None]
    q = np.empty(n)
    todo = np.arange(n)
    while len(todo):
        x4 = g.uniform(0.0, 1.0, len(todo))
        x5 = g.uniform(0.0, 0.1, len(todo))
        ok = x5 < x4 * x4 * (1.0 - x4 * x4) ** 3.5
        q[todo[ok]] = x4[ok]
        todo = todo[~ok]
    vesc = np.sqrt(2.0) * (1.0 + r * r) ** -0.25
    vel = _isotropic(g, n) * (q * vesc)[:, None]
    m = np.full(n, mass / n)
    pos -= np.average(pos, axis=0, weights=m)
    vel -= np.average(vel, axis=0, weights=m)
    return pos * a, vel * np.sqrt(G * mass / a), m


def plummer(n: int, seed: int = 1001, a: float = 1.0, mass: float = 1.0, G: float = 1.0,
            rmax: float = 20.0) -> np.ndarray:
    """Plummer sphere (scale radius a, total mass `mass`, equal masses) as Body records."""
    p, v, m = plummer_f64(n, seed, a, mass, G, rmax)
    return _bodies(p, v, m)


def two_plummer(n_each: int = 131072, seed: int = 1002, separation: float = 10.0,
                rel_speed: float = 0.3, impact: float = 2.0, a: float = 1.0,
                mass_each: float = 1.0, rmax: float = 10.0) -> np.ndarray:
    """Two Plummer spheres `separation` apart along x, offset `impact` along y (a grazing
    orbit), approaching each other at `rel_speed`; centre-of-mass frame."""
    p1, v1, m1 = plummer_f64(n_each, seed, a, mass_each, rmax=rmax)
    p2, v2, m2 = plummer_f64(n_each, seed + 7919, a, mass_each, rmax=rmax)
    p1 += [-separation / 2, -impact / 2, 0.0]
    p2 += [separation / 2, impact / 2, 0.0]
    v1 += [rel_speed / 2, 0.0, 0.0]
    v2 += [-rel_speed / 2, 0.0, 0.0]
    return _bodies(np.concatenate([p1, p2]), np.concatenate([v1, v2]), np.concatenate([m1, m2]))


def uniform_cube(n: int = 1 << 20, seed: int = 1003, sigma: float = 0.5) -> np.ndarray:
    """Uniform in [0,1)^3, at rest, masses log-normal(0, sigma) normalised to total 1."""
    g = rng(seed)
    pos = g.uniform(0.0, 1.0, (n, 3))
    m = g.lognormal(0.0, sigma, n)
    m /= m.sum()
    return _bodies(pos, np.zeros((n, 3)), m)


def batch_sizes(count: int = 512, lo: int = 64, hi: int = 8192, seed: int = 1004) -> np.ndarray:
    """System sizes drawn log-uniform in [lo, hi]."""
    g = rng(seed)
    return np.rint(np.exp(g.uniform(np.log(lo), np.log(hi), count))).astype(np.int64)


def batch_plummer(count: int = 512, lo: int = 64, hi: int = 8192, seed: int = 1004,
                  spacing: float = 0.0) -> tuple[np.ndarray, np.ndarray]:
    """Independent Plummer systems; returns (bodies concatenated, offsets[count+1]).
    `spacing` > 0 places system s at x = s*spacing (they never interact anyway)."""
    sizes = batch_sizes(count, lo, hi, seed)
    parts = []
    for s, n in enumerate(sizes):
        b = plummer(int(n), seed=seed * 1000 + s)
        b[:, 0] += s * spacing
        parts.append(b)
    offsets = np.zeros(count + 1, np.int64)
    offsets[1:] = np.cumsum(sizes)
    return np.concatenate(parts), offsets


def disk_halo(n_disk: int = 12_000_000, n_halo: int = 4_777_216, seed: int = 1005,
              r_disk: float = 3.0, z_disk: float = 0.3, a_halo: float = 10.0,
              halo_mass_ratio: float = 5.0, G: float = 1.0, r_halo_max: float = 200.0,
              r_disk_max: float = 40.0) -> np.ndarray:
    """Exponential disk (surface density ~ exp(-R/r_disk), sech^2 vertical profile of
    scale height z_disk) on circular orbits, inside a Hernquist halo of scale a_halo
    sampled by its inverse cumulative mass r = a sqrt(u) / (1 - sqrt(u)). Disk mass 1;
    a halo particle weighs halo_mass_ratio disk particles. Halo velocities are isotropic
    Gaussian with sigma^2 = v_c^2/3 of the total enclosed mass."""
    g = rng(seed)
    md = 1.0 / n_disk
    mh = halo_mass_ratio * md
    M_disk = 1.0
    M_halo = mh * n_halo

    # disk: R ~ Gamma(2, r_disk) (pdf R e^{-R/r_disk}), truncated
    R = np.empty(n_disk)
    todo = np.arange(n_disk)
    while len(todo):
        rr = g.gamma(2.0, r_disk, len(todo))
        ok = rr <= r_disk_max
        R[todo[ok]] = rr[ok]
        todo = todo[~ok]
    phi = g.uniform(0.0, 2.0 * np.pi, n_disk)
    z = z_disk * np.arctanh(np.clip(g.uniform(-1.0, 1.0, n_disk), -0.999999, 0.999999))

    # halo radii (truncated at r_halo_max by redrawing)
    umax = (r_halo_max / (r_halo_max + a_halo)) ** 2
    su = np.sqrt(g.uniform(0.0, umax, n_halo))
    rh = a_halo * su / (1.0 - su)

    def m_enc(r):
        x = r / r_disk
        disk = M_disk * (1.0 - (1.0 + x) * np.exp(-x))
        halo = M_halo * r * r / (r + a_halo) ** 2 * (1.0 + a_halo / r_halo_max) ** 2
        return disk + np.minimum(halo, M_halo)

    rd = np.sqrt(R * R + z * z)
    vc = np.sqrt(G * m_enc(np.maximum(rd, 1e-6)) / np.maximum(rd, 1e-6))
    dpos = np.stack([R * np.cos(phi), R * np.sin(phi), z], axis=1)
    dvel = np.stack([-vc * np.sin(phi) * R / np.maximum(rd, 1e-6),
                     vc * np.cos(phi) * R / np.maximum(rd, 1e-6), np.zeros(n_disk)], axis=1)

    hpos = _isotropic(g, n_halo) * rh[:, None]
    sig = np.sqrt(G * m_enc(np.maximum(rh, 1e-6)) / np.maximum(rh, 1e-6) / 3.0)
    hvel = g.standard_normal((n_halo, 3)) * sig[:, None]

    pos = np.concatenate([dpos, hpos])
    vel = np.concatenate([dvel, hvel])
    m = np.concatenate([np.full(n_disk, md), np.full(n_halo, mh)])
    pos -= np.average(pos, axis=0, weights=m)
    vel -= np.average(vel, axis=0, weights=m)
    return _bodies(pos, vel, m)
