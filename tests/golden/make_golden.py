"""Regenerates the golden fixtures of the exciton path from the FP64 oracle.

Usage: python tests/golden/make_golden.py
Writes tests/golden/<workload>.npz with the seeded inputs' checksum and the oracle's outputs.  The
reference publishes no golden vectors for this path and cannot be run here (it needs Fortran, MPI,
PETSc/SLEPc and MKL), so these fixtures pin the oracle itself against regressions; the GPU parity
tests compare against them as well as against the live oracle.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import wtb_oracle as O  # noqa: E402
from wtb_gb300 import synthetic as S  # noqa: E402


def input_digest(sysm):
    h = hashlib.sha256()
    for a in (sysm.hop, sysm.ihop, sysm.rvec.astype(np.int64), sysm.rlat, np.array([sysm.efermi])):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def make(name):
    sysm, p = S.workload(name)
    r = O.bsesolver(sysm, p)
    spec = O.bsedielraw(r["Ws"], r["acts"], p.ngrid, sysm.rlat, p)
    out = {"digest": np.array(input_digest(sysm)), "E": r["E"], "eigv": r["eigv"],
           "nocpk": r["nocpk"], "V_row0": O.coulomb_table(r["kpt"][:1], r["kpt"], p, sysm.rlat)[0]}
    for c in ("xx", "yy", "zz", "xy", "sp", "sm"):
        out["act_" + c] = r["acts"][c][: p.nev]
    for c in ("xx", "yy", "zz"):
        out["spec_" + c] = spec[c]
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print(name, r["E"])


if __name__ == "__main__":
    for n in ("hex8_6x6", "hex8_24x24"):
        make(n)
