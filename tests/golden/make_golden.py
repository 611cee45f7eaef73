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


def make_fit_target(name="hex8_36x36", r0_true=44.0, noise=1e-3, seed=2024):
    """Target xx absorption spectrum of the fitting case: the oracle's spinf * eps2_xx at the perturbed
    screening length r0_true plus seeded N(0, noise) noise (no imagrenorm)."""
    sysm, p = S.workload(name)
    p.r0 = r0_true
    r = O.bsesolver(sysm, p, dense_solver=False)
    spinf = 2.0 if sysm.systype == "NP" else 1.0
    spec = O.bsedielraw(r["Ws"], r["acts"], p.ngrid, sysm.rlat, p, spinf=spinf)
    p.renorm = False
    spec_raw = O.bsedielraw(r["Ws"], r["acts"], p.ngrid, sysm.rlat, p, spinf=spinf)
    rng = np.random.default_rng(seed)
    target = spec_raw["xx"][:, 2] + rng.normal(0.0, noise, p.numbse)
    np.savez_compressed(os.path.join(HERE, name + "_fit_target.npz"), digest=np.array(input_digest(sysm)),
                        r0_true=np.array(r0_true), E=r["E"], fxx=r["acts"]["xx"][: p.nev], target=target,
                        spec_xx_renorm=spec["xx"][:, 2])
    print(name, "fit target at r0 =", r0_true, r["E"])


def make_next_rows(name="hex8_6x6"):
    """The (f) rows on the small case: the finite-Q spectrum on a Gamma-M path (bsebnds), the same at 3000 K
    with the Bose-Einstein gap correction (bsebndstemp), the temperature solver's energies and summed
    activities at 300 K and 4000 K (bsesolvertemp), the sorted IPA records (spoptics) and the BZ-resolved
    activity (spoptpolbz)."""
    sysm, p = S.workload(name)
    ks = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])
    qpath = O.kpathbse(sysm.rlat, ks, 3)
    out = {"digest": np.array(input_digest(sysm)), "qpath": qpath, "exk": O.bsebnds(sysm, p, qpath),
           "exk_temp": O.bsebndstemp(sysm, p, qpath, 3000.0, "BE", 0.05, 300.0)}
    for T, ta, st, ph in ((300.0, "FA", 0.0, 0.0), (4000.0, "VE", 2.0e-4, 0.02)):
        r = O.bsesolvertemp(sysm, p, T, ta, st, ph)
        out[f"W_{int(T)}"] = r["Ws"]
        out[f"fdeh_{int(T)}"] = r["fdeh"]
        for c in ("xx", "yy", "zz", "sp", "sm"):
            out[f"actsum_{c}_{int(T)}"] = np.array(r["acts"][c].sum())
    kpt = O.monhkhorst_pack(*p.ngrid, p.mshift, sysm.rlat)
    eigv, vec, nocp = O.bands(sysm, p, kpt)
    out["sp_records"] = O.spoptics_records(eigv, kpt, nocp, O.optsp_all(eigv, vec, kpt, sysm, p), p.nv, p.nc)
    out["bz_act"] = O.spoptpolbz(sysm, p)
    np.savez_compressed(os.path.join(HERE, name + "_next_rows.npz"), **out)
    print(name, "next rows: lowest finite-Q", out["exk"][:2, :].T)


if __name__ == "__main__":
    for n in ("hex8_6x6", "hex8_24x24"):
        make(n)
    make_fit_target()
    make_next_rows()
