"""Access to the committed golden fixtures in ``tests/golden/`` (written by
``tests/golden/make_golden.py``): loading, the pair-table encoding and the neighbour-list digest
that both the writer and the tests use."""
from __future__ import annotations

import hashlib
import json
import os
import zlib

import numpy as np

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ("liquid864_melt", "argon864_c1", "mixture864")


def table_rows(table):
    """Pair table {(ti, tj): (eps, sigma, rcut)} as float rows (ti, tj, eps, sigma, rcut)."""
    return np.array([[ti, tj, e, s, rc] for (ti, tj), (e, s, rc) in sorted(table.items())], dtype=np.float64)


def table_from_rows(rows):
    return {(int(r[0]), int(r[1])): (float(r[2]), float(r[3]), float(r[4])) for r in np.asarray(rows)}


def neighbour_digest(off, idx):
    """Per-atom neighbour counts, per-atom CRC-32 and a whole-list SHA-256 of the sorted rows
    (indices as little-endian int32)."""
    n = len(off) - 1
    count = np.diff(np.asarray(off)).astype(np.int32)
    crc = np.zeros(n, dtype=np.uint32)
    sha = hashlib.sha256()
    for i in range(n):
        row = np.sort(np.asarray(idx[off[i]:off[i + 1]], dtype=np.int32)).astype("<i4").tobytes()
        crc[i] = zlib.crc32(row)
        sha.update(row)
    return count, crc, np.frombuffer(sha.digest(), dtype=np.uint8).copy()


def load(name):
    """One fixture: its arrays, plus ``sys`` (the state as the test helpers take it)."""
    with np.load(os.path.join(GOLDEN_DIR, name + ".npz")) as z:
        fx = {k: z[k] for k in z.files}
    fx["sys"] = dict(pos=fx["pos"], vel=fx["vel"], types=fx["types"], masses=fx["masses"], h=fx["h"],
                     table=table_from_rows(fx["table"]))
    return fx


def examples():
    with open(os.path.join(GOLDEN_DIR, "examples.json")) as f:
        return json.load(f)
