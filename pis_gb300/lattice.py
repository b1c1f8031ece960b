"""Initial-state generators: FCC lattices in the sapphire order and seeded Maxwell-Boltzmann
velocities.

* ``fcc_lattice`` reproduces the atom order of the reference's lattice generator
  (src/bin/sapphire/main.rs:17-24, 61-76): cells ix -> iy -> iz, then the basis
  (0,0,0), (0,1/2,1/2), (1/2,0,1/2), (1/2,1/2,0), positions = a * (cell + basis).
* ``maxwell_boltzmann`` draws N(0, sqrt(KB T / m)) components (src/atoms/velocities.rs:17-33)
  from this project's own seeded generator (numpy PCG64 + standard normal), then removes the
  centre-of-mass drift and rescales to T exactly as src/atoms/velocities.rs:35-59 do. The
  reference's own random stream (rand SmallRng + rand_distr Normal) is not reproduced; states
  are exchanged with it through the data file's Velocities section instead.
"""
from __future__ import annotations

import numpy as np

from .atoms import KB_KJPERMOLEKELVIN

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.0, 0.5, 0.5], [0.5, 0.0, 0.5], [0.5, 0.5, 0.0]])


def fcc_lattice(a: float, nx: int, ny: int, nz: int) -> np.ndarray:
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    cells = np.stack([ix.ravel(), iy.ravel(), iz.ravel()], axis=1).astype(np.float64)
    frac = cells[:, None, :] + FCC_BASIS[None, :, :]
    return (a * frac).reshape(-1, 3)


def fcc_lattice_constant(rho: float) -> float:
    """Lattice constant of an FCC crystal with number density rho (4 atoms per cell)."""
    return (4.0 / rho) ** (1.0 / 3.0)


def maxwell_boltzmann(masses_per_atom: np.ndarray, temperature: float, seed: int) -> np.ndarray:
    m = np.asarray(masses_per_atom, dtype=np.float64)
    n = m.shape[0]
    rng = np.random.Generator(np.random.PCG64(seed))
    sigma = np.sqrt(KB_KJPERMOLEKELVIN * temperature / m)
    v = rng.standard_normal((n, 3)) * sigma[:, None]
    # remove_drift: v -= (sum m v) / (sum m)
    total_mass = 0.0
    p = np.zeros(3)
    for i in range(0, n, 65536):
        total_mass += float(np.sum(m[i:i + 65536]))
        p += np.sum(v[i:i + 65536] * m[i:i + 65536, None], axis=0)
    v -= p / total_mass
    # rescale_to_temperature: lambda = sqrt(T / T_current)
    ke = float(np.sum(0.5 * m * np.sum(v * v, axis=1)))
    t_now = 2.0 * ke / (3 * n * KB_KJPERMOLEKELVIN)
    v *= np.sqrt(temperature / t_now)
    return v


def reduced_temperature(t_star: float) -> float:
    """Temperature to feed the reference's KB so that KB * T equals the reduced T*."""
    return t_star / KB_KJPERMOLEKELVIN


def lj_liquid(n_cells: int, rho: float = 0.8442, t_star: float = 0.72, seed: int = 1):
    """FCC start of the reduced-unit LJ liquid benchmark: (positions, velocities, box edge)."""
    a = fcc_lattice_constant(rho)
    pos = fcc_lattice(a, n_cells, n_cells, n_cells)
    vel = maxwell_boltzmann(np.ones(len(pos)), reduced_temperature(t_star), seed)
    return pos, vel, a * n_cells
