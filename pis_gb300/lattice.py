"""Initial-state generators: FCC lattices in the sapphire order and seeded Maxwell-Boltzmann
velocities.

* ``fcc_lattice`` reproduces the atom order of the reference's lattice generator
  (src/bin/sapphire/main.rs:17-24, 61-76): cells ix -> iy -> iz, then the basis
  (0,0,0), (0,1/2,1/2), (1/2,0,1/2), (1/2,1/2,0), positions = a * (cell + basis).
* ``maxwell_boltzmann`` draws N(0, sqrt(KB T / m)) components (src/atoms/velocities.rs:17-33)
  from this project's own seeded generator (SplitMix64 + Box-Muller, in the C++ host library),
  then removes the centre-of-mass drift and rescales to T as src/atoms/velocities.rs:35-59 do.
  The reference's own random stream (rand SmallRng + rand_distr Normal) is not reproduced;
  states are exchanged with it through the data file's Velocities section instead.
"""
from __future__ import annotations

import numpy as np

from .atoms import KB_KJPERMOLEKELVIN  # noqa: F401

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
    """Seeded Maxwell-Boltzmann velocities, drift removed and rescaled to T (the library's
    generator, include/pis_host.h: pis_maxwell_boltzmann)."""
    from .io import maxwell_boltzmann as mb
    return mb(masses_per_atom, temperature, seed)


def reduced_temperature(t_star: float) -> float:
    """Temperature to feed the reference's KB so that KB * T equals the reduced T*."""
    return t_star / KB_KJPERMOLEKELVIN


def lj_liquid(n_cells: int, rho: float = 0.8442, t_star: float = 0.72, seed: int = 1):
    """FCC start of the reduced-unit LJ liquid benchmark: (positions, velocities, box edge)."""
    a = fcc_lattice_constant(rho)
    pos = fcc_lattice(a, n_cells, n_cells, n_cells)
    vel = maxwell_boltzmann(np.ones(len(pos)), reduced_temperature(t_star), seed)
    return pos, vel, a * n_cells
