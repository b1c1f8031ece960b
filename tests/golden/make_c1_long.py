"""Writes ``argon4000_nve1e4.npz``: the oracle's 10^4-step NVE run of the argon case, for the
reference-order GPU test. Run from the repository root:

    python tests/golden/make_c1_long.py

Test infrastructure only. The case is the repo's argon configuration: 4000 Ar atoms on a 10^3
FCC lattice in the reference's lattice order (a = 5.26 A; src/bin/sapphire/main.rs:61-76), LJ
eps = 0.0104, sigma = 3.405, rc = 2.5 sigma, mass 39.948, Maxwell-Boltzmann velocities at 100 K
(seeded; stored here, so the test does not regenerate them), dt = 0.001. The oracle steps it with
its restatement of the reference's serial manager (LJVOffsetManager,
src/potentials/lennard_jones.rs:186-244; verlet_step_nve, src/potentials/potential.rs:15-33) and
records the energies as exact sums (the definition the GPU library's FP64 path uses) and as the
reference's own walk-order sum. A serial FP64 run without fused multiply-adds gives the same bits
on x86 and Arm, so the GPU test compares bit for bit. Ten seconds of the oracle per hundred steps:
the whole run takes several minutes, which is why it is a fixture and not a live comparison.

Arrays: vel0 (4000 x 3), steps, dt, every (record interval), pe (exact, every `every` steps from 0),
ke (exact, same steps), pe_walk (walk-order sum, same steps), sha_pe (SHA-256 of the exact energy of
every step 0..steps as float64), sha_pos, sha_vel (SHA-256 of the final state as float64, x,y,z per
atom).
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
for p in (ROOT, TESTS):
    if p not in sys.path:
        sys.path.insert(0, p)

OUT = os.path.join(HERE, "argon4000_nve1e4.npz")
STEPS = 10000
EVERY = 10
DT = 0.001


def sha(a) -> np.ndarray:
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(a, dtype=np.float64).tobytes()).digest(), np.uint8)


def main():
    import oracle
    from systems import argon, to_oracle
    oracle.build()
    s = argon()
    o = to_oracle(s)
    pe, ke, pw = o.run_nve_exact(DT, STEPS)
    np.savez_compressed(OUT, vel0=s["vel"], steps=np.int64(STEPS), dt=np.float64(DT), every=np.int64(EVERY),
                        pe=pe[::EVERY], ke=ke[::EVERY], pe_walk=pw[::EVERY], sha_pe=sha(pe), sha_pos=sha(o.pos),
                        sha_vel=sha(o.vel))
    print(f"wrote {OUT}: {STEPS} steps, exact pe {pe[0]:.12g} -> {pe[-1]:.12g}")


if __name__ == "__main__":
    main()
