"""Host-side mirrors of the reference's ``Atoms`` and ``SimulationBox`` (state containers).

``Atoms`` follows src/atoms/new.rs:9-17 (N, 1-based type ids, per-type masses, 3 x N
positions / velocities / forces, box); arrays are (N, 3) float64, the same bytes as
nalgebra's column-major Matrix3xX. ``SimulationBox`` follows src/simulation_box.rs:5-69.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

KB_KJPERMOLEKELVIN = 0.0083144621  # src/constants.rs:3


def inverse3(h: np.ndarray) -> np.ndarray:
    """3x3 inverse as adjugate / determinant with first-row cofactor expansion (the form the
    reference's nalgebra try_inverse uses for 3x3, src/simulation_box.rs:13)."""
    m = np.asarray(h, dtype=np.float64)
    m11 = m[1, 1] * m[2, 2] - m[2, 1] * m[1, 2]
    m10 = m[1, 0] * m[2, 2] - m[2, 0] * m[1, 2]
    m12 = m[1, 0] * m[2, 1] - m[2, 0] * m[1, 1]
    det = m[0, 0] * m11 - m[0, 1] * m10 + m[0, 2] * m12
    out = np.empty((3, 3))
    out[0, 0] = m11 / det
    out[0, 1] = (m[0, 2] * m[2, 1] - m[2, 2] * m[0, 1]) / det
    out[0, 2] = (m[0, 1] * m[1, 2] - m[1, 1] * m[0, 2]) / det
    out[1, 0] = -m10 / det
    out[1, 1] = (m[0, 0] * m[2, 2] - m[2, 0] * m[0, 2]) / det
    out[1, 2] = (m[0, 2] * m[1, 0] - m[1, 2] * m[0, 0]) / det
    out[2, 0] = m12 / det
    out[2, 1] = (m[0, 1] * m[2, 0] - m[2, 1] * m[0, 0]) / det
    out[2, 2] = (m[0, 0] * m[1, 1] - m[1, 0] * m[0, 1]) / det
    return out


@dataclass
class SimulationBox:
    h: np.ndarray
    pbc: tuple = (True, True, True)
    h_inv: np.ndarray = field(init=False)

    def __post_init__(self):
        self.h = np.asarray(self.h, dtype=np.float64).reshape(3, 3).copy()
        self.h_inv = inverse3(self.h)

    @staticmethod
    def from_lammps_data(xlo, xhi, ylo, yhi, zlo, zhi, xy=0.0, xz=0.0, yz=0.0) -> "SimulationBox":
        """SimulationBox::from_lammps_data (src/simulation_box.rs:44-65): columns
        (ax,0,0), (xy,ay,0), (xz,yz,az); always periodic."""
        h = np.array([[xhi - xlo, xy, xz], [0.0, yhi - ylo, yz], [0.0, 0.0, zhi - zlo]])
        return SimulationBox(h, (True, True, True))

    def volume(self) -> float:
        m = self.h
        return abs(m[0, 0] * (m[1, 1] * m[2, 2] - m[2, 1] * m[1, 2])
                   - m[0, 1] * (m[1, 0] * m[2, 2] - m[2, 0] * m[1, 2])
                   + m[0, 2] * (m[1, 0] * m[2, 1] - m[2, 0] * m[1, 1]))


class Atoms:
    """The reference's Atoms struct with a version counter so the GPU manager can tell when
    host arrays were modified and a re-upload is needed."""

    def __init__(self, positions, type_ids, masses, sim_box: SimulationBox, velocities=None, forces=None):
        self.positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3).copy()
        n = self.positions.shape[0]
        self.n_atoms = n
        self.type_ids = np.ascontiguousarray(type_ids, dtype=np.int32).reshape(n).copy()
        self.masses = np.ascontiguousarray(masses, dtype=np.float64).copy()
        self.velocities = np.zeros((n, 3)) if velocities is None else np.asarray(velocities, np.float64).reshape(n, 3).copy()
        self.forces = np.zeros((n, 3)) if forces is None else np.asarray(forces, np.float64).reshape(n, 3).copy()
        self.sim_box = sim_box
        self.version = 0

    def touch(self) -> int:
        """Mark host arrays as changed (call after editing them in place)."""
        self.version += 1
        return self.version

    def mass_i(self, i: int) -> float:
        return float(self.masses[self.type_ids[i] - 1])

    def per_atom_mass(self) -> np.ndarray:
        return self.masses[self.type_ids - 1]

    def kinetic_energy(self) -> float:
        return float(np.sum(0.5 * self.per_atom_mass() * np.sum(self.velocities ** 2, axis=1)))

    def temperature(self, kinetic_energy: float) -> float:
        return 2.0 * kinetic_energy / (3 * self.n_atoms * KB_KJPERMOLEKELVIN)

    def virial_tensor(self) -> np.ndarray:
        return self.positions.T @ self.forces

    def pressure(self, kinetic_energy: float) -> float:
        return (2.0 * kinetic_energy + np.trace(self.virial_tensor())) / (3.0 * self.sim_box.volume())
