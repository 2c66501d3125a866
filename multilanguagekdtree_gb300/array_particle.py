"""Body records and seeded initial conditions.

Mirror of the reference's ``array_particle`` module (MarkCLewis/MultiLanguageKDTree
Parallel/RustVersion/src/array_particle.rs): the ``Particle`` record as a numpy structured
dtype, ``two_bodies`` and ``circular_orbits``, plus the two synthetic workloads the GPU path
is measured on (a thin ring around a central mass and a Plummer sphere).  Every generator
takes a seed; the reference's ``fastrand`` is unseeded, so its outputs cannot be replayed.
"""
from __future__ import annotations

import numpy as np

from ._lib import PARTICLE_DTYPE

__all__ = ["PARTICLE_DTYPE", "empty", "two_bodies", "circular_orbits", "ring", "plummer",
           "to_arrays"]


def empty(n: int) -> np.ndarray:
    return np.zeros(n, dtype=PARTICLE_DTYPE)


def two_bodies() -> np.ndarray:
    """array_particle.rs:10-17: a unit mass at the origin and a 1e-20 mass at x = 1."""
    b = empty(2)
    b[0] = ((0.0, 0.0, 0.0), (0.0, 0.0, 0.0), 1.0, 1.0)
    b[1] = ((1.0, 0.0, 0.0), (0.0, 1.0, 0.0), 1e-4, 1e-20)
    return b


def circular_orbits(n: int, seed: int = 0) -> np.ndarray:
    """array_particle.rs:19-44: n+1 bodies; body 0 is a unit mass at rest at the origin,
    body i+1 orbits at d = 0.1 + 5i/n with angle theta ~ U[0, 6.28), z = 0, speed sqrt(1/d),
    mass 1e-14, radius 1e-7."""
    rng = np.random.default_rng(seed)
    b = empty(n + 1)
    b["r"][0] = 0.00465047
    b["m"][0] = 1.0
    i = np.arange(n, dtype=np.float64)
    d = 0.1 + (i * 5.0 / float(n))
    v = np.sqrt(1.0 / d)
    th = rng.random(n) * 6.28
    b["p"][1:, 0] = d * np.cos(th)
    b["p"][1:, 1] = d * np.sin(th)
    b["v"][1:, 0] = -v * np.sin(th)
    b["v"][1:, 1] = v * np.cos(th)
    b["m"][1:] = 1e-14
    b["r"][1:] = 1e-7
    return b


def ring(n: int, seed: int = 0) -> np.ndarray:
    """Thin ring of n bodies in total: body 0 has mass 1 at the origin at rest; bodies
    1..n-1 have mass 1e-14, radius r ~ U[0.8, 1.2], angle phi ~ U[0, 2 pi),
    z ~ Normal(mean 0, standard deviation 1e-4), and the circular speed sqrt(1/r) of G = 1
    around the central mass, tangential."""
    rng = np.random.default_rng(seed)
    b = empty(n)
    b["m"][0] = 1.0
    b["r"][0] = 0.00465047
    k = n - 1
    if k > 0:
        r = rng.uniform(0.8, 1.2, k)
        phi = rng.uniform(0.0, 2.0 * np.pi, k)
        z = rng.normal(0.0, 1e-4, k)
        v = np.sqrt(1.0 / r)
        c, s = np.cos(phi), np.sin(phi)
        b["p"][1:, 0] = r * c
        b["p"][1:, 1] = r * s
        b["p"][1:, 2] = z
        b["v"][1:, 0] = -v * s
        b["v"][1:, 1] = v * c
        b["m"][1:] = 1e-14
        b["r"][1:] = 1e-7
    return b


def plummer(n: int, seed: int = 0, rmax: float = 20.0) -> np.ndarray:
    """Plummer sphere (G = 1, total mass 1, scale radius 1), equal masses 1/n.

    Radii by the inverse cumulative mass profile r = (U^(-2/3) - 1)^(-1/2), rejected above
    rmax; isotropic directions; speeds v = q * v_esc(r) with q drawn by von Neumann rejection
    from g(q) = q^2 (1 - q^2)^(7/2) (Aarseth, Henon & Wielen 1974); isotropic velocity
    directions; the centre of mass is moved to rest at the origin."""
    rng = np.random.default_rng(seed)
    r = np.empty(0)
    while r.size < n:
        u = rng.random(2 * (n - r.size) + 16)
        u = u[u > 0.0]
        rr = 1.0 / np.sqrt(u ** (-2.0 / 3.0) - 1.0)
        r = np.concatenate([r, rr[rr <= rmax]])
    r = r[:n]

    def iso(count):
        cth = rng.uniform(-1.0, 1.0, count)
        ph = rng.uniform(0.0, 2.0 * np.pi, count)
        sth = np.sqrt(1.0 - cth * cth)
        return np.stack([sth * np.cos(ph), sth * np.sin(ph), cth], axis=1)

    q = np.empty(0)
    while q.size < n:
        m = 2 * (n - q.size) + 16
        x = rng.random(m)
        y = rng.random(m) * 0.1
        q = np.concatenate([q, x[y < x * x * (1.0 - x * x) ** 3.5]])
    q = q[:n]
    vesc = np.sqrt(2.0) * (1.0 + r * r) ** -0.25
    b = empty(n)
    pos = iso(n) * r[:, None]
    vel = iso(n) * (q * vesc)[:, None]
    pos -= pos.mean(axis=0)
    vel -= vel.mean(axis=0)
    b["p"] = pos
    b["v"] = vel
    b["m"] = 1.0 / n
    b["r"] = 0.0
    return b


def to_arrays(b: np.ndarray):
    """(positions (n,3), velocities (n,3), masses (n,)) views/copies of a body array."""
    return np.ascontiguousarray(b["p"]), np.ascontiguousarray(b["v"]), np.ascontiguousarray(b["m"])
