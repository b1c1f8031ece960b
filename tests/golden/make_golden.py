"""Writes the golden fixtures of this directory. Run from the repository root:

    python tests/golden/make_golden.py

Test infrastructure only. Each ``*.npz`` fixture holds a small seeded state and the CPU oracle's
FP64 answers for it (forces, energy, virial, neighbour sets, a short NVE trajectory), so that
the parity tests can check the CUDA path against committed numbers on a machine without the
oracle's sources or the reference's files. ``examples.json`` holds known answers taken from the
reference's example inputs (``example/data.txt``, ``example/data_run.txt``,
``example/example.txt``, ``example/example2.txt``, ``example/argon4000.txt``): the parsed pair
tables with the PairCoeffs quirk, the oracle's energy and forces on the two small files, and the
FCC order, shell count and lattice energy of the argon files. Those inputs are read from the
reference sources (the directory in ``PIS_REFERENCE_DIR``; there is no default); the script refuses to write if they are absent or if the oracle disagrees
with a closed form, so a fixture never records an unpinned oracle.

Fixture arrays (float64 unless noted):
  pos, vel, types (int32), masses, h, table (rows ti, tj, eps, sigma, rcut)
  dt, steps, skin                         run parameters of the trajectory and list
  pe0, force0, ke0, virial0               compute_potential on the input (LJVOffsetManager,
                                          lennard_jones.rs:186-244; virial = sum_i r_i F_i^T,
                                          properties.rs:49-51)
  nl_count (int32), nl_crc (uint32), nl_sha (uint8[32])
                                          full neighbour list at rc (lennard_jones.rs:345-415):
                                          per-atom counts, per-atom CRC-32 of the sorted
                                          int32 indices, SHA-256 of all sorted rows
  pe_steps, ke_steps                      run_nve: energies before step 1 and after each step
                                          (potential.rs:15-33, simulation.rs:8-39)
  pos_end, vel_end                        state after ``steps`` steps
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

from golden_data import FIXTURES, neighbour_digest, table_rows  # noqa: E402

REFERENCE_DIR = os.environ.get("PIS_REFERENCE_DIR", "")


def oracle_answers(sysd, dt, steps, skin):
    from systems import to_oracle
    o = to_oracle(sysd)
    pe0 = o.compute_potential()
    out = dict(pos=sysd["pos"], vel=sysd["vel"], types=np.asarray(sysd["types"], np.int32),
               masses=np.asarray(sysd["masses"], np.float64), h=np.asarray(sysd["h"], np.float64),
               table=table_rows(sysd["table"]), dt=np.float64(dt), steps=np.int64(steps), skin=np.float64(skin),
               pe0=np.float64(pe0), force0=o.force.copy(), ke0=np.float64(o.kinetic_energy()),
               virial0=o.virial_tensor())
    out["nl_count"], out["nl_crc"], out["nl_sha"] = neighbour_digest(*o.full_list())
    if steps:
        pe, ke = o.run_nve(dt, steps)
        out.update(pe_steps=pe, ke_steps=ke, pos_end=o.pos.copy(), vel_end=o.vel.copy())
    return out


def fixtures():
    """The fixture states: the same seeded systems the parity tests build, at 864 atoms."""
    from systems import argon, liquid, melted

    def displaced(sysd, frac, seed):
        rng = np.random.default_rng(seed)
        out = dict(sysd)
        a = sysd["h"][0, 0] / round((len(sysd["pos"]) / 4) ** (1 / 3))
        out["pos"] = np.mod(sysd["pos"] + rng.normal(0, frac * a, sysd["pos"].shape), sysd["h"][0, 0])
        return out

    # reduced LJ liquid (rho* 0.8442, T* 0.72, rc 2.5), melted for 300 steps by the oracle
    liq = melted(liquid(nc=6), steps=300, dt=0.005)
    yield "liquid864_melt", liq, 0.005, 100, 0.3

    # argon (a = 5.26, eps 0.0104, sigma 3.405, rc 8.5125, 100 K), displaced 3 % of a
    ar = displaced(argon(nc=6), 0.03, 5)
    yield "argon864_c1", ar, 0.001, 100, 0.3 * 3.405

    # two types with per-pair cutoffs (types drawn per atom), displaced 2 % of a
    rng = np.random.default_rng(4)
    mix = liquid(nc=6, rho=0.8)
    mix["types"] = rng.integers(1, 3, len(mix["pos"])).astype(np.int32)
    mix["masses"] = np.array([1.0, 2.0])
    mix["table"] = {(1, 1): (1.0, 1.0, 2.5), (2, 2): (0.8, 1.1, 2.75), (1, 2): (0.9, 1.05, 2.6)}
    mix = displaced(mix, 0.02, 2)
    yield "mixture864", mix, 0.005, 50, 0.3


def _sha256(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def _json_table(table):
    return [[ti, tj, e, s, rc] for (ti, tj), (e, s, rc) in sorted(table.items())]


def example_answers():
    """Known answers from the reference's example inputs, each checked against a closed form
    or an independent manager of the oracle before it is recorded."""
    import oracle
    from oracle.data_file import lattice_energy_per_atom
    from pis_gb300.lattice import fcc_lattice

    def path(name):
        p = os.path.join(REFERENCE_DIR, "example", name)
        if not os.path.exists(p):
            raise SystemExit(f"reference example {p} not found: set PIS_REFERENCE_DIR to the reference sources")
        return p

    out = {}
    # data.txt: two argon atoms 4.5 A apart in a 5 A box (min-image separation 0.5 A); one cell
    # per axis, so only the all-pairs manager's answer is meaningful (lennard_jones.rs:62-99)
    p = path("data.txt")
    d = oracle.read_data(p)
    s = oracle.System.from_data(d)
    rij = s.min_image(s.pos[1] - s.pos[0])
    pe = s.compute_potential(manager=oracle.ALLPAIRS)
    u, f = oracle.lj_pair(0.238, 3.405, 8.5, rij)
    assert np.allclose(rij, [-0.5, 0.0, 0.0], rtol=0, atol=1e-15) and pe == u
    assert np.array_equal(s.force[0], -f) and np.array_equal(s.force[1], f)
    out["data.txt"] = dict(sha256=_sha256(p), n_atoms=d["n_atoms"], table=_json_table(d["table"]),
                           box=[d["xlo"], d["xhi"], d["ylo"], d["yhi"], d["zlo"], d["zhi"]],
                           masses=list(map(float, d["masses"])), type_ids=list(map(int, d["type_ids"])),
                           positions=np.asarray(d["positions"]).tolist(), min_image_rij=rij.tolist(),
                           pe_allpairs=pe, forces_allpairs=s.force.tolist())

    # data_run.txt: two types; the "1 2 eps sigma rc" row is read as the single-type form and
    # overwrites (1,1) (commands.rs:262-272); no (1,2) entry, so cross pairs are skipped
    # (lennard_jones.rs:216-222). 3 cells per axis at the largest cutoff: the production
    # half-shell manager is exact and must agree with all pairs.
    p = path("data_run.txt")
    d = oracle.read_data(p)
    assert d["table"] == {(1, 1): (2.0, 0.6, 1.1), (2, 2): (0.8, 1.2, 3.0)}
    s = oracle.System.from_data(d)
    assert s.divide_into_cells(s.max_rcut()) == (3, 3, 3)
    pe = s.compute_potential(manager=oracle.OFFSET)
    f_off = s.force.copy()
    s2 = oracle.System.from_data(d)
    pe_all = s2.compute_potential(manager=oracle.ALLPAIRS)
    assert pe == pe_all and np.array_equal(f_off, s2.force)
    out["data_run.txt"] = dict(sha256=_sha256(p), n_atoms=d["n_atoms"], table=_json_table(d["table"]),
                               box=[d["xlo"], d["xhi"], d["ylo"], d["yhi"], d["zlo"], d["zhi"]],
                               masses=list(map(float, d["masses"])), type_ids=list(map(int, d["type_ids"])),
                               positions=np.asarray(d["positions"]).tolist(),
                               start_velocities=bool(d["start_velocities"]), pe=pe, forces=f_off.tolist())

    # example.txt (500 atoms) and argon4000.txt (4000 atoms): the FCC lattice a = 5.41 in the
    # sapphire order (bin/sapphire/main.rs:61-76), eps 0.238, sigma 3.405, rc 8.5: 54 neighbours
    # per atom (4 shells), zero force, lattice energy per atom in closed form
    for name, nc in (("example.txt", 5), ("argon4000.txt", 10)):
        p = path(name)
        d = oracle.read_data(p)
        gen = fcc_lattice(5.41, nc, nc, nc)
        dev = float(np.abs(np.asarray(d["positions"]) - gen).max())
        assert d["n_atoms"] == 4 * nc ** 3 and dev <= 1e-12
        assert d["table"] == {(1, 1): (0.238, 3.405, 8.5)}
        s = oracle.System.from_data(d)
        pe = s.compute_potential(manager=oracle.OFFSET)
        closed = lattice_energy_per_atom(5.41, 0.238, 3.405, 8.5)
        assert abs(pe / s.n - closed) <= 1e-11 * abs(closed)
        off, _ = s.full_list()
        assert np.all(np.diff(off) == 54)
        out[name] = dict(sha256=_sha256(p), n_atoms=d["n_atoms"], lattice_a=5.41, cells=nc,
                         table=_json_table(d["table"]), max_dev_from_generator=dev,
                         neighbours_per_atom=54, pe=pe, pe_per_atom_closed_form=closed,
                         max_abs_force=float(np.abs(s.force).max()))
    # example2.txt: the same 500-atom lattice with no PairCoeffs section, so the table comes from
    # the input's pair_style / pair_coeff (system.rs:120-168) and the data file's manager is empty
    p = path("example2.txt")
    d = oracle.read_data(p)
    gen = fcc_lattice(5.41, 5, 5, 5)
    dev = float(np.abs(np.asarray(d["positions"]) - gen).max())
    assert d["n_atoms"] == 500 and dev <= 1e-12 and d["table"] == {} and d["start_velocities"]
    out["example2.txt"] = dict(sha256=_sha256(p), n_atoms=d["n_atoms"], lattice_a=5.41, cells=5, table=[],
                               max_dev_from_generator=dev, masses=list(map(float, d["masses"])))
    return out


def main():
    import oracle
    oracle.build()
    ex = example_answers()
    with open(os.path.join(HERE, "examples.json"), "w") as f:
        json.dump(ex, f, indent=1, sort_keys=True)
        f.write("\n")
    for name, sysd, dt, steps, skin in fixtures():
        assert name in FIXTURES
        ans = oracle_answers(sysd, dt, steps, skin)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **ans)
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith((".npz", ".json")):
            print(f"{fn}: {os.path.getsize(os.path.join(HERE, fn))} bytes")


if __name__ == "__main__":
    main()
