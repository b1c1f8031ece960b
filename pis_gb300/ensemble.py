"""Thermostat state of the reference's NVT ensemble, for callers that step an ``Atoms`` through
``LJGpuManager.verlet_step_nvt_nhc``.

``NHThermostatChain`` follows src/ensemble/nvt.rs literally: chain length 3 as
``new_from_args`` builds it (:99-112), masses q_i = KB T tau^2 / 10^i (:37-42), forces
(:59-70), the half step that assigns xi from the current forces rather than integrating it
(:72-80; eta is never advanced), the thermostat's kinetic and potential energy (:82-97) and the
linear target-temperature ramp (:114-124).
"""
from __future__ import annotations

import math

from .atoms import KB_KJPERMOLEKELVIN as KB


class NHThermostatChain:
    def __init__(self, start_temperature: float, end_temperature: float, tau: float, chain_size: int = 3,
                 name: str = "", group: str = "all"):
        self.name, self.group = name, group
        self.chain_size = chain_size
        self.start_temperature = float(start_temperature)
        self.end_temperature = float(end_temperature)
        self.target_temperature = float(start_temperature)
        self.xi = [0.0] * chain_size
        self.eta = [0.0] * chain_size
        self.g = [0.0] * chain_size
        q_value = KB * self.target_temperature * (tau * tau)
        self.q = []
        p = 1.0
        for _ in range(chain_size):
            self.q.append(q_value / p)
            p = p * 10.0

    def compute_forces(self, kinetic_energy: float, n_atoms: int) -> None:
        self.g[0] = 2.0 * kinetic_energy - float(n_atoms * 3) * KB * self.target_temperature
        for j in range(1, self.chain_size):
            self.g[j] = self.q[j - 1] * (self.xi[j - 1] * self.xi[j - 1]) - KB * self.target_temperature

    def propagate_half_step(self, timestep: float) -> None:
        j = self.chain_size - 1
        self.xi[j] = 0.5 * timestep * self.g[j] / self.q[j]
        for l in range(j - 1, -1, -1):
            self.xi[l] = (0.5 * timestep * self.g[l] / self.q[l]) * math.exp(-0.25 * timestep * self.xi[l + 1])

    def kinetic_energy(self) -> float:
        e = 0.0
        for q, x in zip(self.q, self.xi):
            e += 0.5 * q * (x * x)
        return e

    def potential_energy(self, n_atoms: int) -> float:
        e = float(n_atoms * 3) * KB * self.target_temperature * self.eta[0]
        for i in range(1, self.chain_size):
            e += KB * self.target_temperature * self.eta[i]
        return e

    def calculate_target_temperature(self, current_timestep: int, total_timesteps: int) -> None:
        self.target_temperature = (self.start_temperature
                                   + ((self.end_temperature - self.start_temperature) / float(total_timesteps))
                                   * float(current_timestep))
