"""Operator applications of the reference's eigensolve, measured -- TEST INFRASTRUCTURE ONLY.

The reference solves the dense BSE matrix with SLEPc Krylov-Schur (src/module_slepc_solver.F90:29-74):
EPS_HEP, smallest magnitude, tol 1e-8 (relative residual), ncv = nev + mpd with mpd = nev for nev < 1000,
max_it 200.  SLEPc 3.22.2 is not vendored and is absent here, so its count of matrix-vector products is
measured with ARPACK's implicitly restarted Lanczos (scipy.sparse.linalg.eigsh, which='SA' -- the same as
smallest magnitude for these positive spectra; the implicit restart is mathematically equivalent to the
Krylov-Schur restart) with the same nev, ncv and tol, on the oracle's FP64 factored operator (the matrix of
the reference's element-by-element build).  The median over three random start vectors is recorded.

The timed CPU legs of bench.py multiply a sampled dense-matvec time by this count.

Usage: python oracle/krylov_count.py [workload ...]   (writes oracle/krylov_counts.json)
"""
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from oracle import wtb_oracle as O  # noqa: E402
from wtb_gb300 import synthetic as S  # noqa: E402

OUT = os.path.join(HERE, "krylov_counts.json")


def count(name, seeds=(101, 102, 103)):
    import scipy
    import scipy.sparse.linalg as sla

    g_path = os.path.join(ROOT, "tests", "golden", name + "_oracle.npz")
    if os.path.exists(g_path):
        sysm = S.system_from_arrays(np.load(g_path))
        _, p = S.workload(name, params_only=True)
    else:
        sysm, p = S.workload(name)
    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, _ = O.bands(sysm, p, kpt)
    V = O.coulomb_table(kpt, kpt, p, sysm.rlat)
    dim, nev = p.dim, p.nev
    ncv = nev + nev  # ncv = nev + mpd, mpd = nev (src/module_slepc_solver.F90:29-40)
    calls = [0]

    def mv(x):
        calls[0] += x.size // dim
        return O.bse_matvec_factored(x.reshape(dim, -1), eigv, vec, kpt, p, sysm.rlat, V).reshape(x.shape)

    op = sla.LinearOperator((dim, dim), dtype=np.complex128, matvec=mv, matmat=mv)
    runs = []
    for sd in seeds:
        rng = np.random.default_rng(sd)
        v0 = rng.normal(size=dim) + 1j * rng.normal(size=dim)
        calls[0] = 0
        t0 = time.time()
        E = sla.eigsh(op, k=nev, which="SA", tol=1e-8, ncv=ncv, v0=v0, maxiter=200 * dim,
                      return_eigenvectors=False)
        runs.append({"seed": sd, "matvecs": calls[0], "seconds": round(time.time() - t0, 1),
                     "lowest": float(np.min(E))})
        print(name, runs[-1], flush=True)
    mvs = sorted(r["matvecs"] for r in runs)
    return {"nev": nev, "ncv": ncv, "tol": 1e-8, "which": "SA", "dim": dim, "matvecs": int(mvs[len(mvs) // 2]),
            "runs": runs, "solver": f"ARPACK (scipy {scipy.__version__} eigsh) on the FP64 factored operator"}


if __name__ == "__main__":
    names = sys.argv[1:] or ["hex12_60x60", "cubic16_16x16x16"]
    data = json.load(open(OUT)) if os.path.exists(OUT) else {}
    for n in names:
        data[n] = count(n)
    with open(OUT, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
        f.write("\n")
