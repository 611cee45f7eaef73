"""CPU FP64 gradient oracle for the exciton path -- TEST INFRASTRUCTURE ONLY.

Reverse-mode derivatives of L(E, f) = sum_n a_n E_n + b_n f_n (E_n the lowest exciton energies, f_n the
xx activities |sum_j A(j,n) hrx(j)|^2) with respect to the tight-binding hoppings H(R) (hop, ihop) and the
R_0 screening length of V2DRK, written with dense numpy linear algebra on the forward of ``wtb_oracle``
(eigsys -> bands -> bse_build -> eigh -> optsp_all).  Used by ``tests/`` only, as the checker of the
library's wtb_bse_backward.  The reference has no gradients; what is differentiated is the reference's
forward arithmetic (src/module_hamiltonian.F90:200-320, src/module_bse.F90:24-83, :201-245,
src/module_coulomb.F90:286-350, src/module_optics.F90:12-167).

Parity status: pinned by central finite differences of ``wtb_oracle``'s forward itself
(tests/test_oracle_grad.py), not by reference outputs (the reference computes no gradient).

Derivation (dL = Re sum conj(G) dz defines the gradient G of a complex variable z):
  * exciton level: y_n = sum_m A_m Gamma_mn - 2 b_n s_n lambda_n with Gamma_nn = a_n,
    Gamma_mn = -2 b_n s_n conj(s_m)/(E_m - E_n) over the other computed excitons, and lambda_n the solution
    of (H - E_n) lambda_n = P conj(hx) orthogonal to all computed excitons; then dL = Re sum_n y_n^H dH A_n
    and dL/dhx = hbar = sum_n 2 b_n s_n conj(A_n).
  * bands: the BSE kernel V(k,k') <c_k|c'_k'> <v_k|v'_k'> gives the band-vector gradients through
    T_A = V Z(A), T_y = V Z(y); the diagonal E_c - E_v and the velocity elements give the rest.
  * per k: eigenvector back-propagation with the first-component-real gauge (the gauge of ZHEEV('L')),
    Hbar = U conj(B) U^H, B_ab = (conj(K_ab) + i Im(K_bb) U_0a/U_0b)/(lam_b - lam_a), B_bb = Ebar_b,
    K = U^H Ubar, folded onto the lower triangle ZHEEV reads.
  * Fourier: H(k) = sum_R e^{i phi} (hop + i ihop)/ndegen and dH/dk_x = sum_R i R_x e^{i phi} (...)/ndegen.
"""
from __future__ import annotations

import numpy as np

from . import wtb_oracle as O

F32 = np.float32


def forward(sysm, p):
    """Forward pass with everything the backward needs (dense BSE, all its eigenpairs)."""
    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    nk, w = len(kpt), sysm.w90basis
    eall = np.empty((nk, w))
    vall = np.empty((nk, w, w), complex)
    nocp = np.empty(nk, int)
    for k in range(nk):
        e, v, no = O.eigsys(kpt[k], sysm)
        eall[k], vall[k], nocp[k] = e, v, no
    nv, nc = p.nv, p.nc
    if np.any(nocp < nv) or np.any(w - nocp < nc):
        raise O.OracleError("band window outside the occupied/empty states")
    eigv = np.stack([eall[k, nocp[k] - nv:nocp[k] + nc] for k in range(nk)])
    vec = np.stack([vall[k, nocp[k] - nv:nocp[k] + nc] for k in range(nk)])
    H = O.bse_build(eigv, vec, kpt, p, sysm.rlat)
    Ew, Aw = np.linalg.eigh(H)
    E, A = Ew[:p.nev], Aw[:, :p.nev]
    hx = O.optsp_all(eigv, vec, kpt, sysm, p)[0]
    s = A.T @ hx
    return dict(kpt=kpt, eall=eall, vall=vall, nocp=nocp, eigv=eigv, vec=vec, H=H, E=E, A=A, hx=hx, s=s,
                f=np.abs(s) ** 2)


def loss(sysm, p, a, b):
    d = forward(sysm, p)
    return float(np.dot(a, d["E"]) + np.dot(b, d["f"]))


def dV_dr0(kpt, p, rlat):
    """d V2DRK / d r0 = -V q e^{-q w} / eps(q) (zero below KTOL, as V)."""
    if p.coultype != "V2DRK":
        return np.zeros((len(kpt), len(kpt)))
    k1, k2 = kpt[:, None, :], kpt[None, :, :]
    q = O._modk(k1, k2)
    small = q < p.ktol
    q = np.where(small, 1.0, q)
    V = O.coulomb_table(kpt, kpt, p, rlat)
    epar, et, eb = p.ediel[1], p.ediel[0], p.ediel[2]
    eta, kappa = np.sqrt(epar / p.ez), np.sqrt(epar * p.ez)
    pb, pt = (eb - kappa) / (eb + kappa), (et - kappa) / (et + kappa)
    aux1 = (1.0 - (pb * pt * np.exp(-2.0 * q * eta * p.lc))) * kappa
    aux2 = (1.0 - (pt * np.exp(-eta * q * p.lc))) * (1.0 - (pb * np.exp(-eta * q * p.lc)))
    ew = aux1 / aux2 + p.r0 * q * np.exp(-q * p.w_coul)
    return np.where(small, 0.0, -V * q * np.exp(-q * p.w_coul) / ew)


def backward(sysm, p, a, b, d=None):
    """Returns (dL/dhop, dL/dihop, dL/dr0, forward dict) for L = a.E + b.f."""
    d = forward(sysm, p) if d is None else d
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    kpt, eall, vall, nocp, eigv, vec = d["kpt"], d["eall"], d["vall"], d["nocp"], d["eigv"], d["vec"]
    E, A, hx, s = d["E"], d["A"], d["hx"], d["s"]
    nk, nv, nc, nev, w = len(kpt), p.nv, p.nc, p.nev, sysm.w90basis
    nb, dim = nv + nc, nk * nc * nv
    # exciton level
    P = np.eye(dim) - A @ A.conj().T
    lam = np.zeros((dim, nev), complex)
    for n in range(nev):
        M = P @ (d["H"] - E[n] * np.eye(dim)) @ P + A @ A.conj().T
        lam[:, n] = np.linalg.solve(M, P @ np.conj(hx))
    G = np.zeros((nev, nev), complex)
    for n in range(nev):
        for m in range(nev):
            if m == n:
                G[m, n] = a[n]
            elif abs(E[m] - E[n]) > 1e-9 * max(1.0, abs(E[n])):
                G[m, n] = -2 * b[n] * s[n] * np.conj(s[m]) / (E[m] - E[n])
    y = A @ G - 2 * b[None, :] * s[None, :] * lam
    hbar = (2 * b[None, :] * s[None, :] * np.conj(A)).sum(1)
    # band level
    V = O.coulomb_table(kpt, kpt, p, sysm.rlat)
    C, Vb = vec[:, nv:], vec[:, :nv]
    XA, Xy = A.reshape(nk, nc, nv, nev), y.reshape(nk, nc, nv, nev)
    ZA = np.einsum("kco,kvp,kcvn->kopn", C, Vb, XA)
    Zy = np.einsum("kco,kvp,kcvn->kopn", C, Vb, Xy)
    TA = np.einsum("kq,qopn->kopn", V, ZA)
    Ty = np.einsum("kq,qopn->kopn", V, Zy)
    U = np.einsum("kcvn,kopn->kcvop", np.conj(Xy), TA) + np.einsum("kcvn,kopn->kcvop", np.conj(XA), Ty)
    cbar = np.einsum("kvp,kcvop->kco", np.conj(Vb), U)
    vbar = np.einsum("kco,kcvop->kvp", np.conj(C), U)
    de = eigv[:, nv:][:, :, None] - eigv[:, :nv][:, None, :]
    s32 = float(F32(p.cshift))
    phi = de / (de * de + s32 * s32)
    dphi = (s32 * s32 - de * de) / (de * de + s32 * s32) ** 2
    hb = hbar.reshape(nk, nc, nv)
    g = np.real(np.einsum("kcvn,kcvn->kcv", np.conj(Xy), XA))
    Ebar = np.zeros((nk, nb))
    Mbar = np.zeros((nk, w, w), complex)
    for k in range(nk):
        M = O.hlm(kpt[k], sysm)[0]
        Mv = Vb[k] @ M.T
        MHc = C[k] @ np.conj(M)
        cmv = np.conj(C[k]) @ Mv.T
        for c in range(nc):
            for v in range(nv):
                cbar[k, c] += np.conj(hb[k, c, v]) * phi[k, c, v] * Mv[v]
                vbar[k, v] += hb[k, c, v] * phi[k, c, v] * MHc[c]
                gg = g[k, c, v] + np.real(np.conj(hb[k, c, v]) * cmv[c, v]) * dphi[k, c, v]
                Ebar[k, nv + c] += gg
                Ebar[k, v] -= gg
                Mbar[k] += hb[k, c, v] * phi[k, c, v] * np.outer(C[k, c], np.conj(Vb[k, v]))
    Ubar = np.concatenate([vbar, cbar], axis=1)
    # per k and Fourier
    dhop = np.zeros_like(sysm.hop)
    dihop = np.zeros_like(sysm.ihop)
    rv, rl = sysm.rvec, sysm.rlat
    phase = O._phases_f32(kpt, rv, rl)
    Rx = (rv[:, 0] * rl[0, 0] + rv[:, 1] * rl[1, 0] + rv[:, 2] * rl[2, 0]).astype(F32).astype(np.float64)
    nd = sysm.ffactor.astype(np.float64)
    onsite = np.flatnonzero(np.all(rv == 0, axis=1))
    for k in range(nk):
        Uk = vall[k].T
        lamk = eall[k] - np.where(np.arange(w) >= nocp[k], sysm.scs, 0.0)
        b0 = nocp[k] - nv
        Ub = np.zeros((w, w), complex)
        Ea = np.zeros(w)
        Ub[:, b0:b0 + nb] = Ubar[k].T
        Ea[b0:b0 + nb] = Ebar[k]
        K = np.conj(Uk).T @ Ub
        B = np.zeros((w, w), complex)
        for ia in range(w):
            for ib in range(w):
                if ia == ib:
                    B[ia, ib] = Ea[ib]
                    continue
                dl = lamk[ib] - lamk[ia]
                if abs(dl) < 1e-12:
                    continue
                B[ia, ib] = (np.conj(K[ia, ib]) + 1j * K[ib, ib].imag * Uk[0, ia].real / Uk[0, ib].real) / dl
        Hb = Uk @ np.conj(B) @ np.conj(Uk).T
        Gk = np.tril(Hb, -1) + np.conj(np.triu(Hb, 1)).T + np.diag(np.real(np.diag(Hb)))
        e = np.exp(1j * phase[k]) / nd
        dhop += np.real(np.conj(Gk)[None] * e[:, None, None])
        dihop += np.real(np.conj(Gk)[None] * 1j * e[:, None, None])
        fM = 1j * Rx * e
        th = np.real(np.conj(Mbar[k])[None] * fM[:, None, None])
        ti = np.real(np.conj(Mbar[k])[None] * 1j * fM[:, None, None])
        for r in onsite:
            np.fill_diagonal(th[r], 0.0)
            np.fill_diagonal(ti[r], 0.0)
        dhop += th
        dihop += ti
    dV = dV_dr0(kpt, p, sysm.rlat)
    Yd = np.einsum("kco,kvp,kopn->kcvn", np.conj(C), np.conj(Vb), np.einsum("kq,qopn->kopn", dV, ZA))
    dr0 = float(np.real(np.sum(np.conj(y) * Yd.reshape(dim, nev))))
    return dhop, dihop, dr0, d


def spectrum_loss(E, f, dimse, p, vc, target, spinf=1.0):
    """L = sum_j (spinf eps2_xx(omega_j) - target_j)^2 with eps2 of optdiel_grid (rows past nev zero)."""
    Ws = np.zeros(dimse)
    Ws[:len(E)] = E
    fx = np.zeros(dimse)
    fx[:len(f)] = f
    N = int(p.numbse)
    j = np.arange(N, dtype=np.float64)
    elux = p.ebse0 + ((p.ebsef - p.ebse0) * j) / (float(N) - 1.0)
    _, e2 = O.optdiel_grid(1, vc, p.ngrid, elux, Ws, fx, p.cshift)
    r = spinf * e2 - target
    return float(np.sum(r * r))
