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


def system_arrays(sysm):
    """The seeded system itself, stored beside the results: the generator bisects the gap with LAPACK, whose
    last bits may differ between machines, so the full-size tests rebuild the system from these arrays."""
    return {"hop": sysm.hop, "ihop": sysm.ihop, "rvec": sysm.rvec.astype(np.int32),
            "ffactor": sysm.ffactor.astype(np.int32), "rlat": sysm.rlat, "efermi": np.array(sysm.efermi),
            "scs": np.array(sysm.scs), "systype": np.array(sysm.systype)}


def make_fullsize(name, ncv_factor=4, tol=1e-10):
    """Lowest nev excitons of a full-size workload from the oracle's FP64 factored operator
    (bse_matvec_factored: the matrix of the reference's element-by-element build, never formed) under
    ARPACK's implicitly restarted Lanczos (which='SA', tol 1e-10), standing in for SLEPc Krylov-Schur.
    Two runs from different start vectors must agree to 1e-9 eV and every residual ||Hx - Ex|| must be
    below 1e-8 eV; then the activities (dielbsev/dielbsep) and the three bsedielraw spectra."""
    import time

    import scipy.sparse.linalg as sla

    sysm, p = S.workload(name)
    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, nocpk = O.bands(sysm, p, kpt)
    V = O.coulomb_table(kpt, kpt, p, sysm.rlat)
    hrx, hry, hrz, hrsp, hrsm = O.optsp_all(eigv, vec, kpt, sysm, p)
    dim, nev = p.dim, p.nev

    def mv(x):
        return O.bse_matvec_factored(x.reshape(dim, -1), eigv, vec, kpt, p, sysm.rlat, V).reshape(x.shape)

    op = sla.LinearOperator((dim, dim), dtype=np.complex128, matvec=mv, matmat=mv)
    runs = []
    for seed in (1, 2):
        v0 = np.random.default_rng(seed).normal(size=dim) + 1j * np.random.default_rng(seed + 10).normal(size=dim)
        t0 = time.time()
        E, A = sla.eigsh(op, k=nev, which="SA", tol=tol, ncv=ncv_factor * nev, v0=v0)
        o = np.argsort(E)
        runs.append((E[o], A[:, o]))
        print(f"{name}: ARPACK run {seed}: {time.time() - t0:.1f} s, E = {E[o]}")
    E, A = runs[0]
    assert np.max(np.abs(runs[1][0] - E)) < 1e-9, runs[1][0] - E
    res = np.linalg.norm(mv(A) - A * E[None, :], axis=0)
    assert res.max() < 1e-8, res
    Ws = np.zeros(dim)
    Ws[:nev] = E
    acts = {"xx": O.dielbsev(A, hrx, dim), "yy": O.dielbsev(A, hry, dim), "zz": O.dielbsev(A, hrz, dim),
            "xy": O.dielbsep(A, hrx, hry, dim), "xz": O.dielbsep(A, hrx, hrz, dim),
            "yz": O.dielbsep(A, hry, hrz, dim), "sp": O.dielbsev(A, hrsp, dim), "sm": O.dielbsev(A, hrsm, dim)}
    spec = O.bsedielraw(Ws, acts, p.ngrid, sysm.rlat, p)
    out = {"digest": np.array(input_digest(sysm)), "E": E, "residual": res, "eigv_min_gap": np.array(
        np.min(np.diff(E))), **system_arrays(sysm)}
    for c in ("xx", "yy", "zz", "xy", "xz", "yz", "sp", "sm"):
        out["act_" + c] = acts[c][:nev]
    for c in ("xx", "yy", "zz"):
        out["spec_" + c] = spec[c]
    np.savez_compressed(os.path.join(HERE, name + "_oracle.npz"), **out)
    print(name, "residuals", res.max(), "smallest gap", np.min(np.diff(E)))


def lowest_factored(sysm, p, nev, tol=1e-10):
    """Lowest nev excitons (energies, vectors) of the FP64 factored operator under ARPACK, with the bands."""
    import scipy.sparse.linalg as sla

    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, _ = O.bands(sysm, p, kpt)
    V = O.coulomb_table(kpt, kpt, p, sysm.rlat)
    dim = p.dim

    def mv(x):
        return O.bse_matvec_factored(x.reshape(dim, -1), eigv, vec, kpt, p, sysm.rlat, V).reshape(x.shape)

    op = sla.LinearOperator((dim, dim), dtype=np.complex128, matvec=mv, matmat=mv)
    v0 = np.random.default_rng(5).normal(size=dim) + 0.5j
    E, A = sla.eigsh(op, k=nev, which="SA", tol=tol, ncv=max(4 * nev, 20), v0=v0)
    o = np.argsort(E)
    E, A = E[o], A[:, o]
    res = np.linalg.norm(mv(A) - A * E[None, :], axis=0)
    assert res.max() < 1e-8, res
    return E, A, res


def make_batch_subset():
    """Three systems of the 64-system strained batch (the smallest, a middle and the largest BSE dimension):
    their lowest 6 excitons from the FP64 factored operator under ARPACK (tol 1e-10)."""
    batch = S.strained_batch(nsys=64)
    dims = np.array([p.dim for _, p in batch])
    order = np.argsort(dims, kind="stable")
    pick = sorted({int(order[0]), int(order[len(order) // 2]), int(order[-1])})
    out = {"systems": np.array(pick)}
    for i in pick:
        sysm, p = batch[i]
        E, _, res = lowest_factored(sysm, p, p.nev)
        out[f"E_{i}"] = E
        out[f"dim_{i}"] = np.array(p.dim)
        out[f"digest_{i}"] = np.array(input_digest(sysm))
        print("batch system", i, "dim", p.dim, "E", E, "residual", res.max())
    np.savez_compressed(os.path.join(HERE, "batch64_subset_oracle.npz"), **out)


def make_grad_c5(name="hex8_36x36", nentries=24, h=1e-6, seed=77):
    """The differentiation form at its own size (dim 5184, lowest 4): the FP64 gradient oracle's
    (oracle/wtb_oracle_grad.py) gradients with respect to every H(R) entry and r0 of five losses -- each of the
    lowest 4 exciton energies and the L2 spectrum loss against the fitting case's target spectrum -- and
    central differences (step h = 1e-6) of the oracle's forward for the same five losses on a seeded sample
    of H(R) entries and on r0.  The forward of the differences is the factored operator under ARPACK at
    machine precision (energies and xx activities of the lowest 4)."""
    import copy
    import time

    import scipy.sparse.linalg as sla

    from oracle import wtb_oracle_grad as OG

    sysm, p = S.workload(name)
    target = np.load(os.path.join(HERE, name + "_fit_target.npz"))["target"]
    vc = O.vcell3D(sysm.rlat)
    spinf = 2.0 if sysm.systype == "NP" else 1.0
    nev = p.nev
    t0 = time.time()
    d = OG.forward(sysm, p)
    print("forward", time.time() - t0, "E", d["E"])

    def loss_spec(E, f):
        return OG.spectrum_loss(E, f, p.dim, p, vc, target, spinf)

    # cotangents of the spectrum loss in (E, f): central differences of the scalar loss of 2 nev numbers
    gE, gf = np.zeros(nev), np.zeros(nev)
    for n in range(nev):
        for arr, g in ((d["E"], gE), (d["f"], gf)):
            hh = 1e-6 * max(1.0, abs(arr[n]))
            ap, am = arr.copy(), arr.copy()
            ap[n] += hh
            am[n] -= hh
            lp = loss_spec(ap, d["f"]) if arr is d["E"] else loss_spec(d["E"], ap)
            lm = loss_spec(am, d["f"]) if arr is d["E"] else loss_spec(d["E"], am)
            g[n] = (lp - lm) / (2 * hh)
    cot = {f"E{n}": (np.eye(nev)[n], np.zeros(nev)) for n in range(nev)}
    cot["spec"] = (gE, gf)
    out = {"digest": np.array(input_digest(sysm)), "E": d["E"], "f": d["f"], "target": target,
           "spec_loss": np.array(loss_spec(d["E"], d["f"])), "gE_spec": gE, "gf_spec": gf, **system_arrays(sysm)}
    for key, (a, b) in cot.items():
        t0 = time.time()
        dh, di, dr, _ = OG.backward(sysm, p, a, b, d=d)
        out[f"dhop_{key}"], out[f"dihop_{key}"], out[f"dr0_{key}"] = dh, di, np.array(dr)
        print("backward", key, time.time() - t0, "dr0", dr)

    def fwd(s, q):
        kpt = O.monhkhorst_pack(q.ngrid[0], q.ngrid[1], q.ngrid[2], q.mshift, s.rlat)
        eigv, vec, _ = O.bands(s, q, kpt)
        V = O.coulomb_table(kpt, kpt, q, s.rlat)
        hx = O.optsp_all(eigv, vec, kpt, s, q)[0]
        dim = q.dim

        def mv(x):
            return O.bse_matvec_factored(x.reshape(dim, -1), eigv, vec, kpt, q, s.rlat, V).reshape(x.shape)

        op = sla.LinearOperator((dim, dim), dtype=np.complex128, matvec=mv, matmat=mv)
        v0 = np.random.default_rng(3).normal(size=dim) + 0.25j
        E, A = sla.eigsh(op, k=nev, which="SA", tol=0, ncv=24, v0=v0)
        o = np.argsort(E)
        E, A = E[o], A[:, o]
        f = np.abs(A.T @ hx) ** 2
        return np.concatenate([E, [loss_spec(E, f)]])

    rng = np.random.default_rng(seed)
    entries = []
    while len(entries) < nentries:
        which = "hop" if len(entries) % 2 == 0 else "ihop"
        r, m, n = int(rng.integers(sysm.nvec)), int(rng.integers(sysm.w90basis)), int(rng.integers(sysm.w90basis))
        if (which, r, m, n) not in entries:
            entries.append((which, r, m, n))
    fd = np.zeros((nentries + 1, nev + 1))
    t0 = time.time()
    for i, (which, r, m, n) in enumerate(entries):
        sp, sm = copy.deepcopy(sysm), copy.deepcopy(sysm)
        getattr(sp, which)[r, m, n] += h
        getattr(sm, which)[r, m, n] -= h
        fd[i] = (fwd(sp, p) - fwd(sm, p)) / (2 * h)
    pp, pm = copy.deepcopy(p), copy.deepcopy(p)
    pp.r0 += h
    pm.r0 -= h
    fd[nentries] = (fwd(sysm, pp) - fwd(sysm, pm)) / (2 * h)
    print("finite differences", time.time() - t0)
    out["fd_entries"] = np.array([[0 if w == "hop" else 1, r, m, n] for w, r, m, n in entries], dtype=np.int32)
    out["fd"] = fd  # rows: entries then r0; columns: E0..E3, spectrum loss
    out["fd_h"] = np.array(h)
    for i, (which, r, m, n) in enumerate(entries + [("r0", 0, 0, 0)]):
        for j, key in enumerate(list(cot)):
            g = out[f"dr0_{key}"] if which == "r0" else out[f"d{which}_{key}"][r, m, n]
            print(f"{which:4s} {r:2d} {m} {n} {key:5s} grad {float(g): .10e} fd {fd[i, j]: .10e}")
    np.savez_compressed(os.path.join(HERE, name + "_grad_oracle.npz"), **out)


if __name__ == "__main__":
    which = sys.argv[1:] or ["small"]
    if "grad_c5" in which:
        make_grad_c5()
    if "batch64" in which:
        make_batch_subset()
    if "small" in which:
        for n in ("hex8_6x6", "hex8_24x24"):
            make(n)
        make_fit_target()
        make_next_rows()
    for n in ("hex12_60x60", "cubic16_16x16x16"):
        if n in which:
            make_fullsize(n)
