"""Restatement of the reference's LAMMPS-style data-file reader - TEST INFRASTRUCTURE ONLY.

Follows ``run_read_data`` in src/readers/input_file/commands.rs:147-384 of the reference,
including its quirks:

* data files are NOT stripped of inline ``#`` comments (only whole-line comments are
  skipped, :180-182), so trailing comment words are simply extra tokens;
* a ``PairCoeffs`` row whose second token parses as a float - which every integer does - is
  read as the single-type form ``i eps sigma [rcut]`` (:262-272). A two-type row
  ``1 2 eps sigma rcut`` therefore overwrites the (1,1) entry with eps=2, sigma=eps,
  rcut=sigma;
* the default cutoff is 2.5 sigma (:267, :280);
* a ``Velocities`` section switches off Maxwell-Boltzmann initialisation (:194-197);
* errors carry the display strings of src/errors.rs with the 0-based line number that
  ``reader.lines().enumerate()`` gives (:173), and parse errors end with the text Rust's
  ``ParseIntError`` / ``ParseFloatError`` display;
* one deviation: a ``Masses`` row whose type exceeds the declared type count indexes past the
  end of the reference's vector (a panic); here it is an ``InvalidAtomType`` error.
"""
from __future__ import annotations

import math
import re

import numpy as np

_INT_RE = re.compile(r"^[+-]?[0-9]+$")
_FLOAT_RE = re.compile(r"^[+-]?(([0-9]+\.?[0-9]*|\.[0-9]+)([eE][+-]?[0-9]+)?|inf|infinity|nan)$", re.IGNORECASE)


class DataFileError(ValueError):
    pass


def parse_int(tok: str) -> int:
    """Rust ``str::parse::<i32>`` (PisError::IntParseError, src/errors.rs:36-41)."""
    if not _INT_RE.match(tok):
        why = "cannot parse integer from empty string" if not tok else "invalid digit found in string"
        raise DataFileError(f"Error parsing integer number from string {tok}: {why}")
    v = int(tok)
    if v >= 2 ** 31:
        raise DataFileError(f"Error parsing integer number from string {tok}: number too large to fit in target type")
    if v < -(2 ** 31):
        raise DataFileError(f"Error parsing integer number from string {tok}: number too small to fit in target type")
    return v


def parse_float(tok: str) -> float:
    """Rust ``str::parse::<f64>`` (decimal and inf/nan spellings, no hex; PisError::FloatParseError,
    src/errors.rs:29-34)."""
    if not _FLOAT_RE.match(tok):
        why = "cannot parse float from empty string" if not tok else "invalid float literal"
        raise DataFileError(f"Error parsing floating number from string {tok}: {why}")
    return float(tok)


def _usize(v: int, line: int = 0) -> int:
    """``Int32ToUsize::convert_to_usize`` (src/extensions.rs:37-44)."""
    if v < 0:
        raise DataFileError(f"Negative value {v} not allowed on line: {line}")
    return v


def read_data(path: str) -> dict:
    section = ""
    n_atoms = 0
    xlo, xhi, ylo, yhi, zlo, zhi = 0.0, 1.0, 0.0, 1.0, 0.0, 1.0
    masses: list[float] = []
    type_ids = np.zeros(0, dtype=np.int32)
    positions = np.zeros((0, 3))
    velocities = np.zeros((0, 3))
    start_velocities = True
    table: dict[tuple[int, int], tuple[float, float, float]] = {}

    with open(path, "r") as fh:
        lines = fh.read().splitlines()
    for line_num, line in enumerate(lines):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        sp = line.split()
        first = sp[0]
        if first in ("Masses", "Atoms", "PairCoeffs"):
            section = first
            continue
        if first == "Velocities":
            start_velocities = False
            section = first
            continue
        if len(sp) > 1:
            if sp[1] == "atoms":
                n_atoms = _usize(parse_int(sp[0]), line_num)
                type_ids = np.zeros(n_atoms, dtype=np.int32)
                positions = np.zeros((n_atoms, 3))
                velocities = np.zeros((n_atoms, 3))
                continue
            if sp[1] == "atom":
                n_types = _usize(parse_int(sp[0]), line_num)
                masses = (masses + [0.0] * n_types)[:n_types]
                continue
        if len(sp) > 2:
            if sp[2] == "xlo":
                xlo, xhi = parse_float(sp[0]), parse_float(sp[1])
                continue
            if sp[2] == "ylo":
                ylo, yhi = parse_float(sp[0]), parse_float(sp[1])
                continue
            if sp[2] == "zlo":
                zlo, zhi = parse_float(sp[0]), parse_float(sp[1])
                continue

        def req(k):
            if k >= len(sp):
                raise DataFileError(f"Missing argument on line {line_num}")
            return sp[k]

        if section == "Masses":
            t = _usize(parse_int(req(0)), line_num)
            m = parse_float(req(1))
            if t < 1:
                raise DataFileError(f"Atom type {t} out of range")
            if t > len(masses):
                raise DataFileError(f"Atom type {t} out of range")
            masses[t - 1] = m
        elif section == "PairCoeffs":
            i = _usize(parse_int(req(0)), line_num)
            try:
                eps = parse_float(req(1))
                single = True
            except DataFileError:
                single = False
            if single:
                sigma = parse_float(req(2))
                try:
                    rc = parse_float(req(3))
                except DataFileError:
                    rc = 2.5 * sigma
                table[(i, i)] = (eps, sigma, rc)
            else:
                j = _usize(parse_int(req(1)), line_num)
                eps = parse_float(req(2))
                sigma = parse_float(req(3))
                try:
                    rc = parse_float(req(4))
                except DataFileError:
                    rc = 2.5 * sigma
                table[(i, j)] = (eps, sigma, rc)
        elif section == "Atoms":
            aid = _usize(parse_int(req(0)), line_num)
            if aid == 0 or aid > n_atoms:
                raise DataFileError(f"Atom count mismatch: expected {n_atoms}, found {aid}")
            t = _usize(parse_int(req(1)), line_num)
            type_ids[aid - 1] = t
            positions[aid - 1] = [parse_float(req(2)), parse_float(req(3)), parse_float(req(4))]
        elif section == "Velocities":
            aid = _usize(parse_int(req(0)), line_num)
            if aid == 0 or aid > n_atoms:
                raise DataFileError(f"Atom count mismatch: expected {n_atoms}, found {aid}")
            velocities[aid - 1] = [parse_float(req(1)), parse_float(req(2)), parse_float(req(3))]

    return {
        "n_atoms": n_atoms,
        "xlo": xlo, "xhi": xhi, "ylo": ylo, "yhi": yhi, "zlo": zlo, "zhi": zhi,
        "masses": np.array(masses, dtype=np.float64),
        "type_ids": type_ids,
        "positions": positions,
        "velocities": velocities,
        "table": table,
        "start_velocities": start_velocities,
    }


def lattice_energy_per_atom(a: float, eps: float, sigma: float, rc: float, shift: bool = True) -> float:
    """Closed-form LJ energy per atom of a perfect FCC lattice (lattice constant a),
    summing u(r) - u(rc) over every neighbour with r <= rc, halved per pair. Used as a
    known answer for the reference's pair arithmetic (src/potentials/lennard_jones.rs:33-55)."""
    nmax = int(math.ceil(rc / (a / 2.0))) + 1
    basis = [(0, 0, 0), (0, 0.5, 0.5), (0.5, 0, 0.5), (0.5, 0.5, 0)]
    e = 0.0
    ucut = 4 * eps * ((sigma / rc) ** 12 - (sigma / rc) ** 6) if shift else 0.0
    for ix in range(-nmax, nmax + 1):
        for iy in range(-nmax, nmax + 1):
            for iz in range(-nmax, nmax + 1):
                for b in basis:
                    r = a * math.sqrt((ix + b[0]) ** 2 + (iy + b[1]) ** 2 + (iz + b[2]) ** 2)
                    if r == 0.0 or r > rc:
                        continue
                    e += 4 * eps * ((sigma / r) ** 12 - (sigma / r) ** 6) - ucut
    return 0.5 * e
