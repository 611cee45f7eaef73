"""CPU FP64 oracle for the exciton path -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy/scipy, the arithmetic of the reference's exciton path so that the
GPU implementation can be checked against it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may import it; the product path never does.

Parity status: UNPINNED by reference outputs.  The reference ships no tests, no golden vectors and
no expected outputs, and it cannot be compiled here (Fortran, MPI, PETSc/SLEPc and MKL are absent).
The oracle is anchored instead on (a) a line-by-line restatement of the reference routines cited in
each docstring, including their single-precision constants and roundings, (b) analytic known-answer
tests (tests/test_oracle.py), and (c) LAPACK ZHEEV itself (scipy.linalg.lapack.zheev, the same
routine the reference calls for the per-k problem).  Third-party arithmetic the reference links
but does not ship: SLEPc/PETSc 3.22.2 Krylov-Schur (replaced here by dense ``zheevd`` or ARPACK
``eigsh`` on the same matrix) and LAPACK ``ZHEEV`` from MKL/OpenBLAS.

Index conventions (0-based here, 1-based in the reference):
  exciton basis I = k*nc*nv + c*nv + v, c in [0,nc) is band slot nv+c, v in [0,nv) is slot v
  (``quantumnumbers2``, src/module_math.F90:352-379).
"""
from __future__ import annotations

import numpy as np
import scipy.linalg
import scipy.linalg.lapack as lapack

F32 = np.float32
PI_F32 = float(F32(np.arccos(F32(-1.0))))            # acos(-1.) single precision
CIC = -float(F32(F32(0.0904756) * F32(1000.0)))      # -(0.0904756)*10**(3), src/module_coulomb.F90:15
GAMA = float(F32(180.90))                            # e^2/e0, src/module_optics.F90:196
HC = float(F32(19.746e-6))                           # src/module_bse.F90:5111
SQRT2_F32 = float(F32(np.sqrt(F32(2.0))))            # sqrt(2.0) in abscoef, src/module_bse.F90:5113
INV_SQRT2_F32 = float(F32(F32(1.0) / F32(np.sqrt(F32(2.0)))))  # 1.0/sqrt(2.), src/module_bse.F90:2328
RENORM_SHIFT = float(F32(0.15))                      # factor=0.15, src/module_optics.F90:345
ALPHA1_V2DK = float(F32(1.76))                       # src/module_coulomb.F90:17


class OracleError(RuntimeError):
    """Raised where the reference executes STOP."""


# ----------------------------------------------------------------------------- lattice helpers
def prodvec(v1, v2):
    """src/module_math.F90:129-134."""
    return np.array([v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2],
                     v1[0] * v2[1] - v1[1] * v2[0]])


def vcell2D(rlat):
    """|a1 x a2|, src/module_math.F90:143-149."""
    vx = prodvec(rlat[0], rlat[1])
    return float(np.sqrt(vx[0] ** 2 + vx[1] ** 2 + vx[2] ** 2))


def vcell3D(rlat):
    """|(a1 x a2) . a3|, src/module_math.F90:153-160."""
    vx = prodvec(rlat[0], rlat[1])
    return abs(float(vx[0] * rlat[2, 0] + vx[1] * rlat[2, 1] + vx[2] * rlat[2, 2]))


def alat2D(rlat):
    """src/module_math.F90:184-192."""
    s = [float(np.sqrt(np.sum(rlat[i] ** 2))) for i in range(3)]
    return 0.5 * (s[0] + s[1])


def recvec(a1, a2, a3):
    """b_i = 2*pi/vol * (a_j x a_k) with single-precision pi, src/module_kmesh.F90:391-407."""
    v23, v31, v12 = prodvec(a2, a3), prodvec(a3, a1), prodvec(a1, a2)
    vol = abs(a1[0] * v23[0] + a1[1] * v23[1] + a1[2] * v23[2])
    f = (2.0 * PI_F32) / vol
    return f * v23, f * v31, f * v12


def monhkhorst_pack(n1, n2, n3, shift, rlat):
    """Gamma-anchored mesh, i outer, j, l inner (src/module_kmesh.F90:338-386)."""
    b1, b2, b3 = recvec(rlat[0], rlat[1], rlat[2])
    ks = np.array([b1[d] * shift[0] + b2[d] * shift[1] + b3[d] * shift[2] for d in range(3)])
    kpt = np.empty((n1 * n2 * n3, 3))
    c = 0
    for i in range(n1):
        for j in range(n2):
            for l in range(n3):
                for d in range(3):
                    kpt[c, d] = (b1[d] / n1) * i + (b2[d] / n2) * j + (b3[d] / n3) * l + ks[d]
                c += 1
    return kpt


# ----------------------------------------------------------------------------- H(k) and eigsys
def _phases_f32(kpt, rvec, rlat):
    """phi_R = k.R rounded to single precision by cmplx(0.0, ...) (src/module_hamiltonian.F90:240-244).

    kpt (Nk,3) -> (Nk, nR) float64 holding float32 values."""
    Rx = rvec[:, 0] * rlat[0, 0] + rvec[:, 1] * rlat[1, 0] + rvec[:, 2] * rlat[2, 0]
    Ry = rvec[:, 0] * rlat[0, 1] + rvec[:, 1] * rlat[1, 1] + rvec[:, 2] * rlat[2, 1]
    Rz = rvec[:, 0] * rlat[0, 2] + rvec[:, 1] * rlat[1, 2] + rvec[:, 2] * rlat[2, 2]
    kpt = np.atleast_2d(kpt)
    phi = kpt[:, 0:1] * Rx[None] + kpt[:, 1:2] * Ry[None] + kpt[:, 2:3] * Rz[None]
    return phi.astype(F32).astype(np.float64)


def hk_matrix(k, sysm):
    """H(k) = sum_R e^{i phi_R} (H_re + i H_im)(R)/ndegen - E_F I (src/module_hamiltonian.F90:246-259)."""
    phi = _phases_f32(np.asarray(k)[None], sysm.rvec, sysm.rlat)[0]
    e = np.exp(1j * phi)
    H = np.einsum("r,rmn->mn", e / sysm.ffactor.astype(np.float64), sysm.hop + 1j * sysm.ihop)
    H = H - sysm.efermi * np.eye(sysm.w90basis)
    return H


def eigsys(k, sysm, nocp_in=None):
    """One k-point: ZHEEV('V','L') then transpose, nocp, scissor (src/module_hamiltonian.F90:200-320).

    Returns (energias (w,), autovetores (w,w) with row i = eigenvector i, nocp)."""
    H = hk_matrix(k, sysm)
    w, v, info = lapack.zheev(H, compute_v=1, lower=1)
    if info > 0:
        raise OracleError("The algorithm failed to compute eigenvalues.")
    energias = np.array(w, dtype=np.float64)
    autovetores = np.array(v.T)
    pos = np.flatnonzero(energias > 0.0)
    nocp = int(pos[0]) if len(pos) else (sysm.w90basis if nocp_in is None else nocp_in)
    energias[nocp:] += sysm.scs
    return energias, autovetores, nocp


def gauge_fix(vec):
    """Rotate each eigenvector (rows of ``vec``) so its first component is real and >= 0.

    ZHEEV('L') leaves the first component real (ZHETRD('L') keeps e1 invariant); its sign is free
    and every output of the path is invariant under a sign flip, so this is the comparison gauge."""
    v = np.array(vec)
    a = v[..., 0]
    ph = np.where(np.abs(a) > 0, np.conj(a) / np.where(np.abs(a) > 0, np.abs(a), 1.0), 1.0)
    return v * ph[..., None]


def bands(sysm, p, kpt):
    """The eigsys loop of bsesolver (src/module_bse.F90:2230-2245) plus quantumnumbers2's checks.

    Returns eigv (Nk, nv+nc), vector (Nk, nv+nc, w), nocpk (Nk,)."""
    Nk = len(kpt)
    w = sysm.w90basis
    eigv = np.empty((Nk, p.nv + p.nc))
    vec = np.empty((Nk, p.nv + p.nc, w), dtype=np.complex128)
    nocpk = np.empty(Nk, dtype=np.int64)
    for i in range(Nk):
        e, v, nocp = eigsys(kpt[i], sysm)
        nocpk[i] = nocp
        if p.nv > nocp:
            raise OracleError("Number of valence states higher then ocuppied states")
        if p.nc > w - nocp:
            raise OracleError("Number of conduction states higher then unocuppied states")
        eigv[i] = e[nocp - p.nv: nocp + p.nc]
        vec[i] = v[nocp - p.nv: nocp + p.nc]
    return eigv, vec, nocpk


# ----------------------------------------------------------------------------- Coulomb potentials
def _modk(k1, k2):
    """modvec, src/module_math.F90:221-225."""
    d = k1 - k2
    return np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2 + d[..., 2] ** 2)


def coulomb_table(kpt1, kpt2, p, rlat):
    """V(k,k') for every pair, vectorised restatement of module_coulomb (src/module_coulomb.F90).

    Supported: V2DRK (:286-350), V3DL (:98-131), V3D (:64-94), V2DK (:11-60), V2DOH (:354-387),
    V2DT (:135-193), V2DT2 (:243-282), V0DT (:197-238), V1DT (:391-442)."""
    k1 = np.asarray(kpt1)[:, None, :]
    k2 = np.asarray(kpt2)[None, :, :]
    modk = _modk(k1, k2)
    ng = int(p.ngrid[0] * p.ngrid[1] * p.ngrid[2])
    tol = p.ktol
    small = modk < tol
    safe = np.where(small, 1.0, modk)
    ct = p.coultype
    ed = p.ediel
    if ct == "V2DRK":
        vc = vcell2D(rlat)
        vbz = 1.0 / (ng * vc)
        epar, et, eb = ed[1], ed[0], ed[2]
        eta = np.sqrt(epar / p.ez)
        kappa = np.sqrt(epar * p.ez)
        pb = (eb - kappa) / (eb + kappa)
        pt = (et - kappa) / (et + kappa)
        aux1 = (1.0 - (pb * pt * np.exp(-2.0 * safe * eta * p.lc))) * kappa
        aux2 = (1.0 - (pt * np.exp(-eta * safe * p.lc))) * (1.0 - (pb * np.exp(-eta * safe * p.lc)))
        aux3 = p.r0 * safe * np.exp(-safe * p.w_coul)
        ew = (aux1 / aux2) + aux3
        V = (vbz * CIC) * np.exp(-safe * p.w_coul) * (1.0 / ew) * (1.0 / safe)
        return np.where(small, 0.0, V)
    if ct in ("V3DL", "V3D"):
        vc = vcell3D(rlat)
        vbz = 1.0 / (ng * vc)
        e = ed[1] if ct == "V3DL" else 1.0
        V = vbz * (CIC / e) * (1.0 / (safe * safe))
        return np.where(small, 0.0, V)
    if ct == "V2DK":
        a0 = alat2D(rlat)
        vc = vcell2D(rlat)
        r0 = ((ed[1] - 1.0) * p.lc) / (ed[0] + ed[2])
        vbz = 1.0 / (ng * vc)
        g1 = float(p.ngrid[0] * p.ngrid[1])
        auxi = (2.0 * PI_F32 * r0) / (a0 * np.sqrt(g1))
        e = (ed[0] + ed[2]) / 2.0
        v0 = vbz * (CIC / e) * (a0 * np.sqrt(g1) / (2.0 * PI_F32)) * (ALPHA1_V2DK + auxi * 1.0 + 0.0 * auxi ** 2)
        V = vbz * (CIC / e) * (1.0 / (safe * (1 + (r0 * safe))))
        return np.where(small, v0, V)
    if ct == "V2DOH":
        vc = vcell2D(rlat)
        vbz = 1.0 / (ng * vc)
        V = (vbz * CIC) * np.exp(-p.w_coul * safe) * (1.0 / (p.ez * safe))
        return np.where(small, 0.0, V)
    if ct == "V2DT":
        vc = vcell3D(rlat)
        vbz = 1.0 / (ng * vc)
        d = k1 - k2
        gz = np.abs(d[..., 2])
        gpar = np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2)
        rc = 0.5 * rlat[2, 2]
        c1 = (gpar < tol) & (gz < tol)
        c2 = (gpar < tol) & (gz >= tol)
        m2 = np.where(modk > 0, modk, 1.0) ** 2
        v1 = (vbz * CIC) * (-0.5 * rc * rc)
        v2 = (vbz * CIC) * (1.0 / m2) * (1.0 - np.cos(gz * rc) - (gz * rc * np.sin(gz * rc)))
        gp = np.where(gpar > 0, gpar, 1.0)
        aux1 = gz / gp
        aux2 = gpar * rc
        aux3 = gz * rc
        v3 = (vbz * CIC) * (1.0 / m2) * (1.0 + (np.exp(-aux2) * (aux1 * np.sin(aux3) - np.cos(aux3))))
        return np.where(c1, v1, np.where(c2, v2, v3))
    if ct == "V2DT2":
        vc = vcell3D(rlat)
        vbz = 1.0 / (ng * vc)
        d = k1 - k2
        qxy = np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2)
        V = (vbz * CIC) * (1.0 / (safe * safe)) * (1.0 - np.exp(-0.5 * qxy * p.lc) * np.cos(0.5 * p.lc * d[..., 2]))
        return np.where(small, 0.0, V)
    if ct == "V1DT":
        # src/module_coulomb.F90:391-442; J0/J1/K0/K1 (the reference uses Cody's CALJY0/CALJY1/CALCK0/
        # CALCK1, src/module_math.F90:453-1572) and the 100-point trapezoid of integralJ0pot (:429-449)
        import scipy.special as sp
        vc = vcell3D(rlat)
        vbz = 1.0 / (ng * vc)
        d = k1 - k2
        vx = np.abs(d[..., 0])
        qyz = np.sqrt(d[..., 1] * d[..., 1] + d[..., 2] * d[..., 2])
        lc = p.lc
        out = np.empty(modk.shape)
        a = (vx < tol) & (qyz >= tol)
        b = (vx < tol) & (qyz < tol)
        c = ~(a | b)
        out[b] = (vbz * CIC) * ((lc * lc) / 16.0) * (2.0 * np.log(lc) - 1.0)
        if np.any(a):
            out[a] = (vbz * CIC) * np.array([integral_j0_pot(lc, g) for g in qyz[a]])
        if np.any(c):
            x1 = qyz[c] * lc
            x2 = vx[c] * lc
            c1 = qyz[c] * lc * sp.j1(x1) * sp.k0(x2)
            c2 = vx[c] * lc * sp.j0(x1) * sp.k1(x2)
            out[c] = (vbz * CIC) * (1.0 + c1 + c2)
        return out
    if ct == "V0DT":
        vc = vcell3D(rlat)
        vbz = 1.0 / (ng * vc)
        cr = 0.5 * min(float(np.sqrt(np.sum(rlat[i] ** 2))) for i in range(3))
        V = (vbz * CIC) * (1.0 / (safe * safe)) * (1.0 - np.cos(cr * safe))
        return np.where(small, (vbz * CIC) * 0.5 * cr * cr, V)
    raise OracleError("Wrong Coulomb Potential")


def integral_j0_pot(rmax, gperp):
    """integralJ0pot (src/module_math.F90:429-449): trapezoid of r J0(r g) log r on 100 points from eta."""
    import scipy.special as sp
    n = 100
    eta = float(F32(1e-4))
    r = ((np.arange(1, n + 1) - 1.0) / (n - 1.0)) * rmax + eta
    f = r * sp.j0(r * gperp) * np.log(r)
    h = r[1] - r[0]
    res = 0.0
    for i in range(n - 1):
        res = res + (h / 2.0) * (f[i] + f[i + 1])
    return res


# ----------------------------------------------------------------------------- BSE build
def basis(nk, nc, nv):
    """stt of quantumnumbers2: returns (k, c_slot, v_slot) arrays of length dim (0-based slots)."""
    I = np.arange(nk * nc * nv)
    k = I // (nc * nv)
    c = (I // nv) % nc
    v = I % nv
    return k, nv + c, v


def bse_build(eigv, vec, kpt, p, rlat):
    """Dense hbse: upper triangle by matrizelbse (src/module_bse.F90:24-83) then the Hermitian mirror
    (src/module_bse.F90:2392-2415).  Vectorised: element (i,j) is V(k_i,k_j)*<c_i|c_j>*<v_i|v_j>, the
    diagonal is (E_c - E_v) + V(k_i,k_i)."""
    nk = len(kpt)
    kk, cs, vs = basis(nk, p.nc, p.nv)
    V = coulomb_table(kpt, kpt, p, rlat)
    Cv = vec[kk, cs]          # (dim, w)
    Vv = vec[kk, vs]
    gc = np.conj(Cv) @ Cv.T   # <c_i|c_j>
    gv = np.conj(Vv) @ Vv.T   # <v_i|v_j>  (v_i^* . v_j, not the textbook <v_j|v_i>)
    H = V[kk[:, None], kk[None, :]] * gc * gv
    dE = eigv[kk, cs] - eigv[kk, vs]
    d = np.arange(len(kk))
    H[d, d] = dE + V[kk, kk]
    iu = np.triu_indices(len(kk), 1)
    H[iu[1], iu[0]] = np.conj(H[iu[0], iu[1]])
    return H


def kpathbse(rlat, ks, npts):
    """The Q path of bsebnds (src/module_kmesh.F90:124-193): ks (nks, 3) in reduced coordinates, taken in
    pairs (start, end) of segments; returns qpath ((nks//2)*npts, 4) = (normalised path coordinate, Q
    Cartesian)."""
    b1, b2, b3 = recvec(rlat[0], rlat[1], rlat[2])
    ks = np.asarray(ks, dtype=np.float64)
    nks = len(ks)
    ksaux = np.array([[k[0] * b1[d] + k[1] * b2[d] + k[2] * b3[d] for d in range(3)] for k in ks])
    nseg = nks // 2
    kdis = np.empty(nseg)
    kdistot = 0.0
    for i in range(nseg):
        a, b = ksaux[2 * i + 1], ksaux[2 * i]
        kdis[i] = np.sqrt((a[0] - b[0]) ** 2 + (a[1] - b[1]) ** 2 + (a[2] - b[2]) ** 2)   # distvec
        kdistot = kdistot + kdis[i]
    kdis = kdis / kdistot
    q = np.empty((nseg * npts, 4))
    kdisaux = 0.0
    for j in range(nseg):
        for i in range(npts):
            r = j * npts + i
            q[r, 0] = kdisaux + kdis[j] * float(i) / (npts - 1.0)
            for d in range(3):
                q[r, 1 + d] = ksaux[2 * j, d] + (ksaux[2 * j + 1, d] - ksaux[2 * j, d]) * float(i) / (npts - 1.0)
        kdisaux = kdisaux + kdis[j]
    return q


def monhkhorst_packq(q, n1, n2, n3, shift, rlat):
    """The mesh shifted by Q (src/module_kmesh.F90:281-334): q(2:4) + (b1/n1) i + (b2/n2) j + (b3/n3) l +
    kshift, summed in that order."""
    b1, b2, b3 = recvec(rlat[0], rlat[1], rlat[2])
    ks = np.array([b1[d] * shift[0] + b2[d] * shift[1] + b3[d] * shift[2] for d in range(3)])
    out = np.empty((n1 * n2 * n3, 3))
    c = 0
    for i in range(n1):
        for j in range(n2):
            for l in range(n3):
                for d in range(3):
                    out[c, d] = (q[1 + d] + (b1[d] / float(n1)) * float(i) + (b2[d] / float(n2)) * float(j)
                                 + (b3[d] / float(n3)) * float(l) + ks[d])
                c += 1
    return out


def bse_build_q(eigv, vec, eigvq, vecq, kpt, q, p, rlat):
    """Dense finite-Q hbse (matrizelbsekq, src/module_bse.F90:452-569, build loop :1400-1410): conduction
    states from the Q-shifted mesh (eigvq, vecq), valence states from the plain mesh.  Direct term as at
    Q = 0, V(k_i, k_j) <c_i|c_j> <v_i|v_j>, with the diagonal (E_c - E_v) + V(k_i, k_i); for |Q| != 0 the
    exchange term - V(Q, 0) <c_i|v_i> <v_j|c_j> on every element (diagonal included).  The reference fills
    the upper triangle; the Hermitian mirror is returned here."""
    nk = len(kpt)
    kk, cs, vs = basis(nk, p.nc, p.nv)
    V = coulomb_table(kpt, kpt, p, rlat)
    Cv = vecq[kk, cs]
    Vv = vec[kk, vs]
    gc = np.conj(Cv) @ Cv.T
    gv = np.conj(Vv) @ Vv.T
    H = V[kk[:, None], kk[None, :]] * gc * gv
    dE = eigvq[kk, cs] - eigv[kk, vs]
    d = np.arange(len(kk))
    H[d, d] = dE + V[kk, kk]
    modq = np.sqrt(q[1] ** 2 + q[2] ** 2 + q[3] ** 2)
    if modq != 0.0:
        vq = coulomb_table(np.array([q[1:4]]), np.zeros((1, 3)), p, rlat)[0, 0]
        u = np.einsum("iw,iw->i", np.conj(Cv), Vv)           # vcv = <c_i|v_i>; vvc = <v_j|c_j> = conj(u_j)
        H = H - vq * np.outer(u, np.conj(u))
    iu = np.triu_indices(len(kk), 1)
    H[iu[1], iu[0]] = np.conj(H[iu[0], iu[1]])
    return H


def bsebnds(sysm, p, qpath):
    """The Q loop of bsebnds (src/module_bse.F90:1206-1566): for each row of qpath, bands on the Q-shifted
    mesh, the matrizelbsekq matrix and all its eigenvalues (ZHEEV 'N', ascending).  Returns exk (dim, nq)."""
    kpt = monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, nocpk = bands(sysm, p, kpt)
    out = np.empty((p.dim, len(qpath)))
    for i, q in enumerate(qpath):
        kq = monhkhorst_packq(q, p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
        eigvq, vecq, _ = bands(sysm, p, kq)
        H = bse_build_q(eigv, vec, eigvq, vecq, kpt, q, p, sysm.rlat)
        out[:, i] = np.linalg.eigvalsh(H)
    return out


KB_F32 = float(F32(8.617330350e-5))                  # kb = 8.617330350E-5 (single), src/module_math.F90:386


def fermidisteh(ec, ev, temp):
    """f_v - f_c, Fermi level 0; temp = 0 is read as 1E-8 (single) (src/module_math.F90:407-421)."""
    t = float(F32(1e-8)) if temp == 0.0 else temp
    beta = 1.0 / (KB_F32 * t)
    with np.errstate(over="ignore"):
        fv = 1.0 / (np.exp(np.asarray(ev) * beta) + 1.0)
        fc = 1.0 / (np.exp(np.asarray(ec) * beta) + 1.0)
    return fv - fc


def gapcortemp(st, phavg, temp):
    """Varshni-type gap correction (src/module_math.F90:383-391)."""
    aux1 = phavg / ((2.0 * KB_F32) * temp)
    return -st * phavg * (1.0 / np.tanh(aux1) - 1.0)


def gapcortemp2(st, phavg, temp):
    """Bose-Einstein gap correction (src/module_math.F90:395-403)."""
    return -((2.0 * st) / (np.exp(phavg / temp) - 1.0))


def bsesolvertemp(sysm, p, temp, ta="FA", st=0.0, phavg=0.0, dtfull=True, cpol=True):
    """bsesolvertemp (src/module_bse.F90:2649-3263): bands with scs + tcor, the matrizelbsetemp matrix
    (:575-660) completed from its upper triangle as ZHEEV 'U' reads it, E(i,j) = D(i,j) f_min(i,j) and
    E(i,i) = dE_i + V(k_i,k_i) f_i, all eigenpairs, and dielbseptemp's activities (:784-810) of every exciton."""
    import dataclasses
    tcor = {"VE": lambda: gapcortemp(st, phavg, temp), "BE": lambda: gapcortemp2(st, phavg, temp)}.get(ta, lambda: 0.0)()
    s2 = dataclasses.replace(sysm, scs=sysm.scs + tcor)
    kpt = monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, s2.rlat)
    eigv, vec, nocpk = bands(s2, p, kpt)
    hx, hy, hz, hsp, hsm = optsp_all(eigv, vec, kpt, s2, p)
    nk = len(kpt)
    kk, cs, vs = basis(nk, p.nc, p.nv)
    f = fermidisteh(eigv[kk, cs], eigv[kk, vs], temp)
    D = bse_build(eigv, vec, kpt, p, s2.rlat)
    V = coulomb_table(kpt, kpt, p, s2.rlat)
    idx = np.arange(len(kk))
    E = D * f[np.minimum(idx[:, None], idx[None, :])]
    E[idx, idx] = (eigv[kk, cs] - eigv[kk, vs]) + V[kk, kk] * f
    W, A = np.linalg.eigh(E)

    def act(h1, h2):
        s1 = A.T @ h1
        s2_ = A.T @ (h2 * f)
        return (s1 * np.conj(s2_)).real

    z = np.zeros(len(W))
    acts = {"xx": act(hx, hx), "yy": act(hy, hy), "zz": act(hz, hz),
            "xy": act(hx, hy) if dtfull else z, "xz": act(hx, hz) if dtfull else z,
            "yz": act(hy, hz) if dtfull else z, "sp": act(hsp, hsp) if cpol else z, "sm": act(hsm, hsm) if cpol else z}
    return {"Ws": W, "A": A, "acts": acts, "fdeh": f, "E": E, "tcor": tcor}


def bsebndstemp(sysm, p, qpath, temp, ta="FA", st=0.0, phavg=0.0):
    """The Q loop of bsebndstemp (src/module_bse.F90:1572-1990): bsebnds with scs + tcor and
    matrizelbsekqtemp (:664-780), i.e. the finite-Q couplings weighted by f_v - f_c of the row's transition
    (E(i,j) = H(i,j) f_min(i,j), E(i,i) = dE_i + (H(i,i) - dE_i) f_i for the Hermitian completion of the upper
    triangle).  Returns exk (dim, nq)."""
    import dataclasses
    tcor = {"VE": lambda: gapcortemp(st, phavg, temp), "BE": lambda: gapcortemp2(st, phavg, temp)}.get(ta, lambda: 0.0)()
    s2 = dataclasses.replace(sysm, scs=sysm.scs + tcor)
    kpt = monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, s2.rlat)
    eigv, vec, _ = bands(s2, p, kpt)
    nk = len(kpt)
    kk, cs, vs = basis(nk, p.nc, p.nv)
    idx = np.arange(p.dim)
    out = np.empty((p.dim, len(qpath)))
    for i, q in enumerate(qpath):
        kq = monhkhorst_packq(q, p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, s2.rlat)
        eigvq, vecq, _ = bands(s2, p, kq)
        H = bse_build_q(eigv, vec, eigvq, vecq, kpt, q, p, s2.rlat)
        dE = eigvq[kk, cs] - eigv[kk, vs]
        f = fermidisteh(eigvq[kk, cs], eigv[kk, vs], temp)
        E = H * f[np.minimum(idx[:, None], idx[None, :])]
        E[idx, idx] = dE + (H[idx, idx].real - dE) * f
        out[:, i] = np.linalg.eigvalsh(E)
    return out


def spoptpolbz(sysm, p):
    """BZ-resolved optical activity (src/module_bse.F90:4532-4797): per k-point the sums over the nc x nv
    transitions of |h_a|^2, h_a = <c|dH/dk_a|v> / (E_c - E_v + i sme) (optspbz, src/module_optics.F90:257-311,
    then a complex division; sme = CSHIFT in double), the circular |n (h_x +- i h_y)|^2 with n = 1/sqrt(2) in
    single precision, and (sp - sm)/(sp + sm).  Returns act (nk, 6)."""
    kpt = monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, nocpk = bands(sysm, p, kpt)
    act = np.zeros((len(kpt), 6))
    n = INV_SQRT2_F32
    for k in range(len(kpt)):
        dx, dy, dz = hlm(kpt[k], sysm)
        s = np.zeros(5)
        for c in range(p.nc):
            for v in range(p.nv):
                cv, vv = vec[k, p.nv + c], vec[k, v]
                d = (eigv[k, p.nv + c] - eigv[k, v]) + 1j * p.cshift
                hx, hy, hz = [(np.conj(cv) @ (D @ vv)) / d for D in (dx, dy, dz)]
                s += [abs(hx) ** 2, abs(hy) ** 2, abs(hz) ** 2, abs(n * (hx + 1j * hy)) ** 2,
                      abs(n * (hx - 1j * hy)) ** 2]
        act[k, :5] = s
        act[k, 5] = (s[3] - s[4]) / (s[3] + s[4])
    return act


def bse_matvec_factored(x, eigv, vec, kpt, p, rlat, V=None):
    """Matrix-free y = H x through V(k,k') and the orbital factorisation; same operator as bse_build."""
    nk = len(kpt)
    nc, nv = p.nc, p.nv
    w = vec.shape[2]
    if V is None:
        V = coulomb_table(kpt, kpt, p, rlat)
    C = vec[:, nv:nv + nc]        # (nk, nc, w)
    Vb = vec[:, :nv]              # (nk, nv, w)
    nb = x.size // (nk * nc * nv)
    X = x.reshape(nk, nc, nv, nb)
    # Z[k,o,p,b] = sum_{c,v} C[k,c,o] Vb[k,v,p] X[k,c,v,b], as two batched products over k
    U = np.matmul(np.swapaxes(Vb, 1, 2)[:, None], X)                     # (nk, nc, w_p, nb)
    Z = np.matmul(np.swapaxes(C, 1, 2), U.reshape(nk, nc, w * nb))       # (nk, w_o, w_p*nb)
    # T = V Z with V real: one real product on the interleaved re/im panel
    Zr = np.ascontiguousarray(Z).view(np.float64).reshape(nk, -1)
    T = (V @ Zr).view(np.complex128).reshape(nk, w, w, nb)               # (nk, o, p, b)
    # Y[k,c,v,b] = sum_{o,p} conj(C[k,c,o]) conj(Vb[k,v,p]) T[k,o,p,b]
    R = np.matmul(np.conj(C), T.reshape(nk, w, w * nb)).reshape(nk, nc, w, nb)
    Y = np.matmul(np.conj(Vb)[:, None], R)                               # (nk, nc, nv, nb)
    dE = (eigv[:, nv:nv + nc][:, :, None] - eigv[:, :nv][:, None, :])
    Y = Y + dE[..., None] * X
    return Y.reshape(x.shape)


def slepc_solver(HX, NE):
    """Lowest NE eigenpairs of the dense Hermitian HX (stands in for SLEPc Krylov-Schur,
    src/module_slepc_solver.F90:12-97; EPS_SMALLEST_MAGNITUDE equals smallest-algebraic for the
    positive BSE spectra used here).  Returns (EX (NE,), HE (dim, NE))."""
    n = HX.shape[0]
    w, v = scipy.linalg.eigh(HX, subset_by_index=[0, min(NE, n) - 1], driver="evr")
    return w, v


# ----------------------------------------------------------------------------- optics
def hlm(k, sysm):
    """dH/dk_alpha = sum_R i R_alpha e^{i phi_R} H(R)/ndegen, on-site diagonal of H(R=0) removed,
    R_alpha and phi rounded to single precision (src/module_optics.F90:12-108)."""
    rvec, rlat = sysm.rvec, sysm.rlat
    phi = _phases_f32(np.asarray(k)[None], rvec, rlat)[0]
    Rx = (rvec[:, 0] * rlat[0, 0] + rvec[:, 1] * rlat[1, 0] + rvec[:, 2] * rlat[2, 0]).astype(F32).astype(np.float64)
    Ry = (rvec[:, 0] * rlat[0, 1] + rvec[:, 1] * rlat[1, 1] + rvec[:, 2] * rlat[2, 1]).astype(F32).astype(np.float64)
    Rz = (rvec[:, 0] * rlat[0, 2] + rvec[:, 1] * rlat[1, 2] + rvec[:, 2] * rlat[2, 2]).astype(F32).astype(np.float64)
    Hc = (sysm.hop + 1j * sysm.ihop).copy()
    for i in range(len(rvec)):
        if np.all(rvec[i] == 0):
            Hc[i][np.diag_indices(sysm.w90basis)] = 0.0
    e = np.exp(1j * phi) / sysm.ffactor
    hx = np.einsum("r,rmn->mn", 1j * Rx * e, Hc)
    hy = np.einsum("r,rmn->mn", 1j * Ry * e, Hc)
    hz = np.einsum("r,rmn->mn", 1j * Rz * e, Hc)
    return hx, hy, hz


def optsp_all(eigv, vec, kpt, sysm, p):
    """hr_alpha for every basis state (src/module_bse.F90:2317-2348 calling optsp,
    src/module_optics.F90:113-167).  factor = 1./esp is assigned to a real variable, so the scaling is
    Re(1/(E_c - E_v + i*float32(CSHIFT))).  Returns hrx, hry, hrz, hrsp, hrsm (dim,) complex."""
    nk = len(kpt)
    nc, nv = p.nc, p.nv
    dim = nk * nc * nv
    out = np.empty((3, dim), dtype=np.complex128)
    s32 = float(F32(p.cshift))
    for k in range(nk):
        hs = hlm(kpt[k], sysm)
        for c in range(nc):
            for v in range(nv):
                I = k * nc * nv + c * nv + v
                cv = vec[k, nv + c]
                vv = vec[k, v]
                esp = (eigv[k, nv + c] - eigv[k, v]) + 1j * s32
                factor = (1.0 / esp).real
                for a in range(3):
                    out[a, I] = factor * (np.conj(cv) @ (hs[a] @ vv))
    hrsp = (out[0] + 1j * out[1]) * INV_SQRT2_F32
    hrsm = (out[0] - 1j * out[1]) * INV_SQRT2_F32
    return out[0], out[1], out[2], hrsp, hrsm


def dielbsev(A, hopt, dim):
    """act(i) = |sum_j A(j,i) h(j)|^2 for i <= nev, zero beyond (src/module_bse.F90:201-245)."""
    act = np.zeros(dim)
    s = A.T @ hopt
    act[:A.shape[1]] = (s * np.conj(s)).real
    return act


def dielbsep(A, h1, h2, dim):
    """act(i) = Re[(sum A h1)(sum A h2)^*] (src/module_bse.F90:171-196)."""
    act = np.zeros(dim)
    s1 = A.T @ h1
    s2 = A.T @ h2
    act[:A.shape[1]] = (s1 * np.conj(s2)).real
    return act


# ----------------------------------------------------------------------------- spectrum
def avgsme(E):
    """10 * (sum_{i>=2} (E_i - E_{i-1})) / ndim (src/module_optics.F90:313-335)."""
    s = 0.0
    for i in range(1, len(E)):
        s = s + E[i] - E[i - 1]
    return 10.0 * (s / float(len(E)))


def optdiel_grid(rtype, vc, ngrid, elux, E, f, sme):
    """optdiel for a vector of photon energies (src/module_optics.F90:171-255)."""
    baux = float(F32(ngrid[0] * ngrid[1] * ngrid[2])) * vc
    caux = GAMA / (baux * 1.0)
    delta = 1.0 if rtype == 1 else 0.0
    smef = avgsme(E) + sme
    ex = E[None, :]
    el = np.asarray(elux)[:, None]
    eaux = ((el - ex) ** 2) + (smef ** 2)
    rpart = np.sum(f[None, :] * ((ex - el) / eaux), axis=1)
    ipart = np.sum(f[None, :] * (smef / eaux), axis=1)
    return delta + rpart * caux, ipart * caux


def imagrenorm(E1, dielf):
    """In-place baseline renormalisation of dielf[:,2] (src/module_optics.F90:338-401)."""
    aux = E1 - RENORM_SHIFT
    if aux <= 0.0:
        return dielf
    n = dielf.shape[0]
    ibegin = 0
    for i in range(n):
        if dielf[i, 0] <= aux:
            ibegin = i
        else:
            break
    if ibegin + 1 >= n:
        return dielf
    aux3 = dielf[ibegin + 1, 2]
    dielf[: ibegin + 1, 2] = 0.0
    t = dielf[ibegin + 1:, 2] - aux3
    dielf[ibegin + 1:, 2] = np.where(t < 0.0, 0.0, t)
    return dielf


COMPONENTS = ("xx", "yy", "zz", "xy", "xz", "yz")
POL_COMPONENTS = ("xx", "yy", "zz", "sp", "sm")


def dielraw(Ws, acts, comps, rtype1, ngrid, rlat, p, spinf=1.0):
    """optdiel over the given activity columns, then imagrenorm and the spin factor: the common body of
    bsedielraw (src/module_bse.F90:835-1036), bsedielrawpol (:1043-1199), spdielraw (:4090-4308) and
    spdielrawpol (:4318-4524).  ``rtype1`` holds the components optdiel gets with rtype 1."""
    vc = vcell3D(rlat)
    N = int(p.numbse)
    j = np.arange(N, dtype=np.float64)
    elux = p.ebse0 + ((p.ebsef - p.ebse0) * j) / (float(N) - 1.0)
    out = {}
    for comp in comps:
        rtype = 1 if comp in rtype1 else 0
        r, im = optdiel_grid(rtype, vc, ngrid, elux, Ws, acts[comp], p.cshift)
        d = np.stack([elux, r, im], axis=1)
        if p.renorm:
            imagrenorm(Ws[0], d)
        d[:, 1] *= spinf
        d[:, 2] *= spinf
        out[comp] = d
    return out


def bsedielraw(Ws, acts, ngrid, rlat, p, spinf=1.0):
    """epsilon(omega) for the six components (src/module_bse.F90:835-1036).

    ``Ws`` and ``acts`` are the dim-row arrays that bsesolver writes (rows past nev hold E = 0 and
    zero activities).  Returns dict comp -> (numbse, 3) array [omega, spinf*eps1, spinf*eps2]."""
    return dielraw(Ws, acts, COMPONENTS, ("xx", "yy", "zz"), ngrid, rlat, p, spinf)


def bsedielrawpol(Ws, acts, ngrid, rlat, p, spinf=1.0):
    """xx yy zz sp sm, every one with optdiel rtype 1 (src/module_bse.F90:1043-1199)."""
    return dielraw(Ws, acts, POL_COMPONENTS, POL_COMPONENTS, ngrid, rlat, p, spinf)


def spdielraw(esp, acts, ngrid, rlat, p, spinf=1.0):
    """The independent-particle spectrum (src/module_bse.F90:4090-4308): bsedielraw's sums over the
    transitions of spoptics."""
    return dielraw(esp, acts, COMPONENTS, ("xx", "yy", "zz"), ngrid, rlat, p, spinf)


def spdielrawpol(esp, acts, ngrid, rlat, p, spinf=1.0):
    """src/module_bse.F90:4318-4524."""
    return dielraw(esp, acts, POL_COMPONENTS, POL_COMPONENTS, ngrid, rlat, p, spinf)


def bubblem(vec, a):
    """Bubblem(a, b, vec, n) (src/module_math.F90:287-308) literally: for i = 1..n, for j = n..i+1 step -1,
    swap rows j-1 and j when vec(j-1, a) > vec(j, a).  Pure Python, O(n^2): small cases only.  ``a`` is
    0-based here."""
    v = np.array(vec, copy=True)
    n = v.shape[0]
    for i in range(n):
        for j in range(n - 1, i, -1):
            if v[j - 1, a] > v[j, a]:
                t = v[j - 1].copy()
                v[j - 1] = v[j]
                v[j] = t
    return v


def stable_sort_rows(vec, a):
    """The result of Bubblem: a stable ascending sort of the rows by column ``a`` (ties, including -0 and
    +0, keep their order)."""
    return np.asarray(vec)[np.argsort(np.asarray(vec)[:, a], kind="stable")]


def spoptics_records(eigv, kpt, nocpk, hr, nv, nc, f=None):
    """spoptics' vecres(dimsp, 15) in REAL(4) (src/module_bse.F90:4962-4991; bsesolver :2317-2348), sorted
    by Bubblem on column 7 (:4992).  hr = (hrx, hry, hrz, hrsp, hrsm) of optsp_all.  With f (dim,), the
    activity columns times f_v - f_c before the rounding, as bsesolvertemp writes them."""
    F = np.float32
    nk = len(kpt)
    dim = nk * nc * nv
    rec = np.zeros((dim, 15), dtype=F)
    hx, hy, hz, hsp, hsm = hr

    def rp(a, b):
        return (a * np.conj(b)).real

    for k in range(nk):
        for c in range(nc):
            for v in range(nv):
                I = k * nc * nv + c * nv + v
                rec[I, 0:3] = F(kpt[k, 0]), F(kpt[k, 1]), F(kpt[k, 2])
                rec[I, 3] = F(nocpk[k])
                rec[I, 4] = F(nocpk[k] - nv + (nv + c + 1))
                rec[I, 5] = F(nocpk[k] - nv + (v + 1))
                rec[I, 6] = F(eigv[k, nv + c] - eigv[k, v])
                w = 1.0 if f is None else f[I]
                rec[I, 7:15] = [F(rp(hx[I], hx[I]) * w), F(rp(hy[I], hy[I]) * w), F(rp(hz[I], hz[I]) * w),
                                F(rp(hx[I], hy[I]) * w), F(rp(hx[I], hz[I]) * w), F(rp(hy[I], hz[I]) * w),
                                F(rp(hsp[I], hsp[I]) * w), F(rp(hsm[I], hsm[I]) * w)]
    return stable_sort_rows(rec, 6)


def abscoef(e1, e2, efoton):
    """alpha = sqrt(2)*omega/hc*sqrt(|eps| - eps1) (src/module_bse.F90:5107-5114)."""
    aux = np.sqrt(e1 * e1 + e2 * e2)
    return (SQRT2_F32 * efoton) * (1.0 / HC) * np.sqrt(aux - e1)


def optprops(e1, e2, omega):
    """refractive index, extinction, reflectivity, absorption, loss (src/module_bse.F90:5075-5124)."""
    aux = np.sqrt(e1 * e1 + e2 * e2)
    n = np.sqrt((aux + e1) / 2.0)
    kap = np.sqrt((aux - e1) / 2.0)
    refl = ((n - 1.0) ** 2 + kap * kap) / ((n + 1.0) ** 2 + kap * kap)
    return {"refr": n, "ext": kap, "refl": refl, "abs": abscoef(e1, e2, omega),
            "eloss": e2 / (e1 * e1 + e2 * e2)}


# ----------------------------------------------------------------------------- whole path
def bsesolver(sysm, p, dense_solver=True, nev=None, with_vectors=False):
    """The bsesolver path (src/module_bse.F90:2023-2594) for the oracle: mesh -> eigsys -> optics ->
    build -> lowest nev -> oscillator strengths.  Returns a dict with Ws (dim,), acts, E (nev,), A."""
    nev = p.nev if nev is None else nev
    kpt = monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, nocpk = bands(sysm, p, kpt)
    hrx, hry, hrz, hrsp, hrsm = optsp_all(eigv, vec, kpt, sysm, p)
    dim = p.dim
    if dense_solver:
        H = bse_build(eigv, vec, kpt, p, sysm.rlat)
        E, A = slepc_solver(H, nev)
    else:
        import scipy.sparse.linalg as sla
        V = coulomb_table(kpt, kpt, p, sysm.rlat)
        op = sla.LinearOperator((dim, dim), dtype=np.complex128,
                                matvec=lambda x: bse_matvec_factored(x.reshape(-1, 1), eigv, vec, kpt, p,
                                                                     sysm.rlat, V).ravel())
        E, A = sla.eigsh(op, k=nev, which="SA", tol=1e-12)
        o = np.argsort(E)
        E, A = E[o], A[:, o]
    Ws = np.zeros(dim)
    Ws[:nev] = E
    acts = {"xx": dielbsev(A, hrx, dim), "yy": dielbsev(A, hry, dim), "zz": dielbsev(A, hrz, dim),
            "xy": dielbsep(A, hrx, hry, dim), "xz": dielbsep(A, hrx, hrz, dim),
            "yz": dielbsep(A, hry, hrz, dim), "sp": dielbsev(A, hrsp, dim), "sm": dielbsev(A, hrsm, dim)}
    out = {"kpt": kpt, "eigv": eigv, "vec": vec, "nocpk": nocpk, "E": E, "Ws": Ws, "acts": acts,
           "hr": np.stack([hrx, hry, hrz, hrsp, hrsm])}
    if with_vectors:
        out["A"] = A
    return out


def round_f15_4(x):
    """The 7F15.4 text handoff of bse_opt_diel.dat (src/module_bse.F90:2556-2567)."""
    return np.round(np.asarray(x, dtype=np.float64), 4)


# ----------------------------------------------------------------------------- output records
def _fortran_special(x, w):
    s = "NaN" if np.isnan(x) else ("Infinity" if w >= 8 + (x < 0) else "Inf")
    if np.isinf(x) and x < 0:
        s = "-" + s
    return "*" * w if len(s) > w else s.rjust(w)


def fortran_F(x, w, d):
    """Fw.d editing of the binary value x, restated with exact decimal arithmetic: rounded to d decimals
    (nearest, ties to even), right-justified; the optional leading zero dropped when it does not fit; w
    asterisks when the number does not fit."""
    from decimal import ROUND_HALF_EVEN, Decimal
    x = float(x)
    if not np.isfinite(x):
        return _fortran_special(x, w)
    from decimal import localcontext
    with localcontext() as ctx:
        ctx.prec = 1200                            # every double has an exact decimal expansion of < 800 digits
        q = Decimal(x).quantize(Decimal(1).scaleb(-d), rounding=ROUND_HALF_EVEN)
    neg = np.signbit(x)
    mag = format(abs(q), "f")
    if d > 0 and "." not in mag:
        mag += "." + "0" * d
    s = ("-" if neg else "") + mag
    if len(s) > w and mag.startswith("0."):
        s = ("-" if neg else "") + mag[1:]
    return "*" * w if len(s) > w else s.rjust(w)


def fortran_E(x, w, d):
    """Ew.d editing: 0.d1..dd E+xx (the E dropped for a three-digit exponent), d significant digits rounded
    from the exact binary value (nearest, ties to even)."""
    from decimal import ROUND_HALF_EVEN, Decimal
    x = float(x)
    if not np.isfinite(x):
        return _fortran_special(x, w)
    neg = np.signbit(x)
    if x == 0.0:
        digits, e10 = "0" * d, 0
    else:
        from decimal import localcontext
        with localcontext() as ctx:
            ctx.prec = 1200
            dx = abs(Decimal(x))
            e = dx.adjusted()                  # dx = m * 10**e with 1 <= m < 10
            m = (dx.scaleb(-e)).quantize(Decimal(1).scaleb(-(d - 1)), rounding=ROUND_HALF_EVEN)
            if m >= 10:
                m = (m / 10).quantize(Decimal(1).scaleb(-(d - 1)), rounding=ROUND_HALF_EVEN)
                e += 1
        digits = format(m, "f").replace(".", "")[:d].ljust(d, "0")
        e10 = e + 1
    exp = f"E{'-' if e10 < 0 else '+'}{abs(e10):02d}" if abs(e10) <= 99 else f"{'-' if e10 < 0 else '+'}{abs(e10):03d}"
    s = ("-" if neg else "") + "0." + digits + exp
    if len(s) > w:
        s = ("-" if neg else "") + "." + digits + exp
    return "*" * w if len(s) > w else s.rjust(w)


def fortran_I(v, w, m=1):
    """Iw.m editing (Iw.0 of zero is blank)."""
    v = int(v)
    if m == 0 and v == 0:
        return " " * w
    s = str(abs(v)).rjust(m, "0")
    s = ("-" if v < 0 else "") + s
    return "*" * w if len(s) > w else s.rjust(w)


def list_directed_real(x, kind):
    """One real item of a list-directed WRITE as gfortran's runtime edits it (the reference's top-level README
    names the GNU compiler): G editing with scale factor 1P, 1PG25.17E3 for REAL(8) and 1PG16.9E2 for REAL(4)
    (of the single-precision value, as real(x) rounds it).  The G rule of the Fortran standard: with the value
    rounded to d significant digits (nearest, ties to even) and 10**(k-1) <= |r| < 10**k, F(w-n).(d-k) and
    n = e+2 blanks when 0 <= k <= d, else 1PEw.dEe (one digit before the point, d-1 after); zero as
    F(w-n).(d-1) and n blanks.  Exact decimal arithmetic."""
    from decimal import ROUND_HALF_EVEN, Decimal, localcontext
    w, d, e = (25, 17, 3) if kind == 8 else (16, 9, 2)
    x = float(np.float32(x)) if kind == 4 else float(x)
    if not np.isfinite(x):
        return _fortran_special(x, w)
    n = e + 2
    sign = "-" if np.signbit(x) else ""
    if x == 0.0:
        return (sign + "0." + "0" * (d - 1)).rjust(w - n) + " " * n
    with localcontext() as ctx:
        ctx.prec = 1200
        dx = abs(Decimal(x))
        ex = dx.adjusted()
        m = dx.scaleb(-ex).quantize(Decimal(1).scaleb(-(d - 1)), rounding=ROUND_HALF_EVEN)
        if m >= 10:
            m = (m / 10).quantize(Decimal(1).scaleb(-(d - 1)), rounding=ROUND_HALF_EVEN)
            ex += 1
        k = ex + 1
        if 0 <= k <= d:
            q = dx.quantize(Decimal(1).scaleb(-(d - k)), rounding=ROUND_HALF_EVEN)
            mag = format(q, "f")
            if "." not in mag:
                mag += "."
            return (sign + mag).rjust(w - n) + " " * n
        s = sign + format(m, "f") + "E" + ("-" if ex < 0 else "+") + str(abs(ex)).rjust(e, "0")
    return s.rjust(w)


def list_directed_record(items):
    """One list-directed output record as gfortran writes it: a blank before the first item, one blank before
    every later item except a character item that follows a character item; character items as they are,
    4-byte integers as I11, reals by list_directed_real.  items: ("c", str), ("i", int), ("r8", x), ("r4", x).
    A WRITE with no items is an empty record."""
    s, prev_char = "", None
    for t, v in items:
        is_char = t == "c"
        s += " " if prev_char is None or not (is_char and prev_char) else ""
        prev_char = is_char
        s += v if is_char else (fortran_I(v, 11) if t == "i" else list_directed_real(v, 8 if t == "r8" else 4))
    return s


def exclft(sysdim, ngrid, rlat, fosc, enexc):
    """Radiative lifetime (src/module_bse.F90:326-370) with the reference's single-precision constants."""
    cfe, lspd, hbar = float(F32(7.297e-3)), float(F32(299.792e16)), float(F32(6.582e-16))
    ng = float(ngrid[0] * ngrid[1] * ngrid[2])
    with np.errstate(divide="ignore"):
        if sysdim == "3D":
            aux1 = (4.0 * cfe) * (enexc * enexc * enexc)
            aux2 = fosc / ng
            aux3 = 3.0 * (lspd * lspd) * (hbar * hbar * hbar)
            return 1.0 / ((aux1 * aux2) / aux3)
        if sysdim == "2D":
            aux1 = ng * vcell2D(rlat) * hbar
            aux2 = (8.0 * PI_F32 * cfe * enexc) * fosc
            return aux1 / aux2
        if sysdim == "1D":
            aux2 = (2.0 * PI_F32 * cfe * enexc * enexc) * fosc
            aux1 = ng * rlat[0, 0] * hbar * hbar * lspd
            return aux1 / aux2
    raise OracleError("Wrong System dimension")
