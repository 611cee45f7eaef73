"""The FP64 oracle on the CPU: known-answer tests, invariants, the golden fixtures, and the C restatement.

The reference ships no tests or golden outputs for this path; these checks pin the oracle by
(1) single-precision constants and roundings read off the reference sources, (2) analytic known answers
(no Coulomb interaction => excitons are the lowest transition energies; Lorentzian sum rule; gauge
behaviour of eigenvalues versus oscillator strengths), (3) agreement of two independent restatements
(vectorised numpy and the element-by-element C loop), and (4) committed golden fixtures.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import wtb_oracle as O
from wtb_gb300 import synthetic as S

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def small():
    sysm, p = S.workload("hex8_6x6")
    kpt = O.monhkhorst_pack(*p.ngrid, p.mshift, sysm.rlat)
    eigv, vec, nocp = O.bands(sysm, p, kpt)
    return sysm, p, kpt, eigv, vec, nocp


def test_single_precision_constants():
    assert O.CIC == -90.47559356689453
    assert O.PI_F32 == 3.1415927410125732
    assert O.GAMA == 180.89999389648438
    assert O.INV_SQRT2_F32 == 0.7071067690849304
    assert O.RENORM_SHIFT == 0.15000000596046448
    assert O.HC == float(np.float32(19.746e-6))


def test_mesh_is_gamma_anchored_k_outer():
    rlat = S.hex_lattice()
    k = O.monhkhorst_pack(3, 2, 1, (0.0, 0.0, 0.0), rlat)
    assert np.all(k[0] == 0.0)
    b1, b2, _ = O.recvec(*rlat)
    np.testing.assert_allclose(k[1], b2 / 2, atol=1e-15)     # (i=0, j=1): j runs inside i
    np.testing.assert_allclose(k[2], b1 / 3, atol=1e-15)
    np.testing.assert_allclose(k, S.monkhorst_pack((3, 2, 1), rlat), atol=1e-15)
    # reciprocal vectors use single-precision pi: a_i . b_j = 2*pi_f32 delta_ij
    np.testing.assert_allclose(rlat @ np.array([b1, b2, O.recvec(*rlat)[2]]).T, 2 * O.PI_F32 * np.eye(3), atol=1e-12)


def test_eigsys_zheev_gauge_and_occupation(small):
    sysm, p, kpt, eigv, vec, nocp = small
    e, v, n = O.eigsys(kpt[5], sysm)
    assert np.all(np.diff(e) >= 0)
    np.testing.assert_allclose(v @ v.conj().T, np.eye(sysm.w90basis), atol=1e-12)
    assert np.max(np.abs(v[:, 0].imag)) < 1e-12          # first component real (ZHETRD('L') keeps e1)
    assert n == np.sum(e <= 0) == sysm.w90basis // 2
    H = O.hk_matrix(kpt[5], sysm)
    np.testing.assert_allclose(H @ v.T, v.T * e[None, :], atol=1e-11)


def test_scissor_above_fermi_level(small):
    sysm, p, kpt, *_ = small
    s2 = sysm.copy()
    s2.scs = 0.4
    e0, _, n0 = O.eigsys(kpt[3], sysm)
    e1, _, n1 = O.eigsys(kpt[3], s2)
    assert n0 == n1
    np.testing.assert_allclose(e1[:n0], e0[:n0])
    np.testing.assert_allclose(e1[n0:], e0[n0:] + 0.4)


def test_band_window_errors(small):
    sysm, p, kpt, *_ = small
    q = S.BSEParams(**{**p.__dict__})
    q.nv = sysm.w90basis // 2 + 1
    with pytest.raises(O.OracleError, match="valence states higher"):
        O.bands(sysm, q, kpt)
    q = S.BSEParams(**{**p.__dict__})
    q.nc = sysm.w90basis // 2 + 1
    with pytest.raises(O.OracleError, match="conduction states higher"):
        O.bands(sysm, q, kpt)


def test_no_interaction_gives_transition_energies(small):
    """With V = 0 (KTOL larger than every |k - k'|) the excitons are the lowest E_c - E_v."""
    sysm, p, kpt, eigv, vec, _ = small
    q = S.BSEParams(**{**p.__dict__})
    q.ktol = 1e6
    H = O.bse_build(eigv, vec, kpt, q, sysm.rlat)
    E, _ = O.slepc_solver(H, 6)
    kk, cs, vs = O.basis(len(kpt), p.nc, p.nv)
    dE = np.sort(eigv[kk, cs] - eigv[kk, vs])[:6]
    np.testing.assert_allclose(E, dE, atol=1e-12)


def test_hermitian_and_matrix_free_equal_dense(small):
    sysm, p, kpt, eigv, vec, _ = small
    H = O.bse_build(eigv, vec, kpt, p, sysm.rlat)
    assert np.abs(H - H.conj().T).max() == 0.0
    x = np.random.default_rng(3).normal(size=(p.dim, 4)) + 1j
    np.testing.assert_allclose(O.bse_matvec_factored(x, eigv, vec, kpt, p, sysm.rlat), H @ x, atol=1e-12)


def test_phase_gauge_changes_oscillators_not_energies(small):
    """Per-(k, band) phases leave the exciton energies unchanged but change |sum_j A_j h_j|^2
    (no conjugate on A in dielbsev); a sign flip leaves both unchanged."""
    sysm, p, kpt, eigv, vec, _ = small
    rng = np.random.default_rng(9)
    ph = np.exp(1j * rng.uniform(0, 2 * np.pi, vec.shape[:2]))
    vec2 = vec * ph[..., None]
    sgn = np.where(rng.uniform(size=vec.shape[:2]) < 0.5, -1.0, 1.0)
    vec3 = vec * sgn[..., None]
    res = []
    for v in (vec, vec2, vec3):
        H = O.bse_build(eigv, v, kpt, p, sysm.rlat)
        E, A = O.slepc_solver(H, 3)
        h = O.optsp_all(eigv, v, kpt, sysm, p)[0]
        res.append((E, O.dielbsev(A, h, p.dim)[:3]))
    np.testing.assert_allclose(res[1][0], res[0][0], atol=1e-12)
    np.testing.assert_allclose(res[2][0], res[0][0], atol=1e-12)
    np.testing.assert_allclose(res[2][1], res[0][1], rtol=1e-9, atol=1e-14)
    assert np.max(np.abs(res[1][1] - res[0][1])) > 1e-6 * np.max(res[0][1])


def test_optsp_real_part_scaling(small):
    """optsp assigns 1./esp to a real: h = <c|dH|v> * Re(1/(dE + i*CSHIFT_f32))."""
    sysm, p, kpt, eigv, vec, _ = small
    hx = O.optsp_all(eigv, vec, kpt, sysm, p)[0]
    dx, _, _ = O.hlm(kpt[0], sysm)
    c, v = vec[0, p.nv], vec[0, 0]
    de = eigv[0, p.nv] - eigv[0, 0]
    s = float(np.float32(p.cshift))
    np.testing.assert_allclose(hx[0], (np.conj(c) @ dx @ v) * de / (de * de + s * s), rtol=1e-13)


def test_lorentzian_sum_rule():
    """Integral of eps2 over the window equals C * sum_n f_n [atan((b-E_n)/g) - atan((a-E_n)/g)], with the
    width g = CSHIFT + avgsme (renormalisation off)."""
    p = S.BSEParams(ngrid=(4, 4, 1), nc=1, nv=1, numbse=40001, ebse0=-20.0, ebsef=25.0, cshift=0.05, renorm=False)
    rlat = S.hex_lattice()
    Ws = np.array([1.5, 2.0, 2.5])
    f = np.array([1.0, 0.5, 0.25])
    acts = {c: f for c in O.COMPONENTS}
    d = O.bsedielraw(Ws, acts, p.ngrid, rlat, p)["xx"]
    C = O.GAMA / (16 * O.vcell3D(rlat))
    g = p.cshift + O.avgsme(Ws)
    assert abs(g - (0.05 + 10.0 * 1.0 / 3.0)) < 1e-14
    expect = C * np.sum(f * (np.arctan((p.ebsef - Ws) / g) - np.arctan((p.ebse0 - Ws) / g)))
    integral = np.trapezoid(d[:, 2], d[:, 0])
    assert abs(integral - expect) / expect < 1e-6


def test_zero_tail_narrows_the_width():
    """Rows past nev hold E = 0 (quirk of the file handoff): avgsme telescopes to -10 E_1 / dim."""
    Ws = np.zeros(1000)
    Ws[:3] = [1.5, 2.0, 2.5]
    assert abs(O.avgsme(Ws) - (-10.0 * 1.5 / 1000)) < 1e-15


def test_imagrenorm_baseline():
    d = np.zeros((10, 3))
    d[:, 0] = np.linspace(0, 0.9, 10)
    d[:, 2] = np.linspace(1.0, 2.0, 10)
    O.imagrenorm(0.56, d)          # E1 - 0.15_f32 = 0.41 -> last omega below is index 4 (omega = 0.4)
    assert np.all(d[:5, 2] == 0.0)
    np.testing.assert_allclose(d[5:, 2], np.linspace(1.0, 2.0, 10)[5:] - np.linspace(1.0, 2.0, 10)[5])
    d2 = np.ones((5, 3))
    O.imagrenorm(0.1, d2)          # E1 - 0.15 <= 0: untouched
    assert np.all(d2 == 1.0)


def test_bubblem_is_a_stable_sort():
    """Bubblem swaps only on a strictly greater key: its result is the stable ascending sort, with ties
    (including -0 and +0) in their original order."""
    rng = np.random.default_rng(7)
    v = np.zeros((60, 3), dtype=np.float32)
    v[:, 0] = rng.integers(0, 6, 60).astype(np.float32) * np.float32(0.25)
    v[:5, 0] = [0.0, -0.0, 0.0, -0.0, 0.5]
    v[:, 1] = np.arange(60)
    v[:, 2] = rng.standard_normal(60)
    a = O.bubblem(v, 0)
    b = O.stable_sort_rows(v, 0)
    np.testing.assert_array_equal(a, b)
    assert np.all(np.diff(a[:, 0]) >= 0)
    for key in np.unique(v[:, 0]):             # ties keep their input order
        rows = a[a[:, 0] == key, 1]
        assert np.all(np.diff(rows) > 0)


def test_pol_spectrum_shares_the_lorentzian_sum():
    """bsedielrawpol's sp/sm columns get the rtype-1 sum of bsedielraw's xx (eps1 offset 1); spdielraw is
    bsedielraw over the transition list."""
    p = S.BSEParams(ngrid=(4, 4, 1), nc=1, nv=1, numbse=301, ebse0=0.0, ebsef=4.0, cshift=0.05, renorm=True)
    rlat = S.hex_lattice()
    rng = np.random.default_rng(3)
    Ws = np.sort(rng.uniform(1.0, 3.0, 40))
    f = {c: rng.uniform(0.0, 1.0, 40) for c in O.COMPONENTS + ("sp", "sm")}
    six = O.bsedielraw(Ws, f, p.ngrid, rlat, p, spinf=2.0)
    pol = O.bsedielrawpol(Ws, f, p.ngrid, rlat, p, spinf=2.0)
    for c in ("xx", "yy", "zz"):
        np.testing.assert_array_equal(pol[c], six[c])
    same = dict(f, xx=f["sp"])
    np.testing.assert_array_equal(pol["sp"], O.bsedielraw(Ws, same, p.ngrid, rlat, p, spinf=2.0)["xx"])
    off = O.bsedielraw(Ws, dict(f, xy=f["sm"]), p.ngrid, rlat, p, spinf=1.0)["xy"]
    pm = O.bsedielrawpol(Ws, f, p.ngrid, rlat, p, spinf=1.0)["sm"]
    np.testing.assert_allclose(pm[:, 1], off[:, 1] + 1.0, rtol=1e-14)   # rtype 1 vs 0: eps1 offset only
    np.testing.assert_array_equal(pm[:, 2], off[:, 2])
    sp = O.spdielraw(Ws, f, p.ngrid, rlat, p, spinf=2.0)
    for c in O.COMPONENTS:
        np.testing.assert_array_equal(sp[c], six[c])


def test_spoptics_records(small):
    """The IPA records: sorted by transition energy, one per (k, c, v), quantum numbers from nocp, and the
    circular activities obey |h+|^2 + |h-|^2 = 2 s^2 (|hx|^2 + |hy|^2) with s = 1/sqrt(2) in REAL(4)."""
    sysm, p, kpt, eigv, vec, nocp = small
    hr = O.optsp_all(eigv, vec, kpt, sysm, p)
    rec = O.spoptics_records(eigv, kpt, nocp, hr, p.nv, p.nc)
    assert rec.dtype == np.float32 and rec.shape == (p.dim, 15)
    assert np.all(np.diff(rec[:, 6]) >= 0)
    ids = {(int(r[4]) - int(r[3]), int(r[3]) - int(r[5])) for r in rec}
    assert ids == {(c + 1, p.nv - v - 1) for c in range(p.nc) for v in range(p.nv)}
    np.testing.assert_allclose(rec[:, 6].min(), np.float32((eigv[:, p.nv] - eigv[:, p.nv - 1]).min()), rtol=1e-7)
    s2 = O.INV_SQRT2_F32 ** 2
    lhs = rec[:, 13].astype(np.float64) + rec[:, 14]
    rhs = 2.0 * s2 * (rec[:, 7].astype(np.float64) + rec[:, 8])
    np.testing.assert_allclose(lhs, rhs, rtol=1e-5, atol=1e-6 * rhs.max())
    assert np.all(rec[:, 7:10] >= 0)
    assert np.all(rec[:, 10] ** 2 <= rec[:, 7] * rec[:, 8] * (1 + 1e-5) + 1e-12)   # Cauchy-Schwarz


def test_q_mesh_and_path():
    """monhkhorst_packq at Q = 0 is the plain mesh bit for bit (0 + t == t); the path coordinate runs 0..1
    over the segments and each segment interpolates its corner points."""
    rlat = S.hex_lattice()
    kp = O.monhkhorst_pack(4, 3, 1, (0.1, 0.0, 0.0), rlat)
    kq = O.monhkhorst_packq(np.zeros(4), 4, 3, 1, (0.1, 0.0, 0.0), rlat)
    assert np.array_equal(kp, kq)
    q = np.array([0.0, 0.01, -0.02, 0.0])
    np.testing.assert_allclose(O.monhkhorst_packq(q, 4, 3, 1, (0.1, 0.0, 0.0), rlat), kp + q[1:], atol=1e-15)
    ks = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.5, 0.0, 0.0], [1 / 3, 1 / 3, 0.0]])
    path = O.kpathbse(rlat, ks, 5)
    assert path.shape == (10, 4)
    assert path[0, 0] == 0.0 and abs(path[-1, 0] - 1.0) < 1e-15
    assert np.all(np.diff(path[:5, 0]) > 0) and np.all(np.diff(path[5:, 0]) > 0)
    b1, b2, b3 = O.recvec(rlat[0], rlat[1], rlat[2])
    np.testing.assert_allclose(path[4, 1:], 0.5 * b1, atol=1e-15)
    np.testing.assert_allclose(path[9, 1:], (b1 + b2) / 3.0, atol=1e-15)


def test_finite_q_matrix(small):
    """matrizelbsekq: at Q = 0 the plain BSE matrix; for Q != 0 Hermitian, and the exchange part is the rank-1
    term -V(Q,0) u u^H (its one nonzero eigenvalue is -V(Q,0)|u|^2 > 0 for an attractive V)."""
    sysm, p, kpt, eigv, vec, nocp = small
    H0 = O.bse_build(eigv, vec, kpt, p, sysm.rlat)
    Hq0 = O.bse_build_q(eigv, vec, eigv, vec, kpt, np.zeros(4), p, sysm.rlat)
    assert np.array_equal(H0, Hq0)
    q = np.array([0.1, 0.05, 0.02, 0.0])
    kq = O.monhkhorst_packq(q, *p.ngrid, p.mshift, sysm.rlat)
    eq, vq, _ = O.bands(sysm, p, kq)
    Hq = O.bse_build_q(eigv, vec, eq, vq, kpt, q, p, sysm.rlat)
    np.testing.assert_allclose(Hq, np.conj(Hq.T), atol=1e-14)
    # the direct part alone: the same shifted conduction states with |Q| read as zero
    Hd = O.bse_build_q(eigv, vec, eq, vq, kpt, np.array([0.1, 0.0, 0.0, 0.0]), p, sysm.rlat)
    ev = np.linalg.eigvalsh(Hq - Hd)
    vQ = O.coulomb_table(np.array([q[1:]]), np.zeros((1, 3)), p, sysm.rlat)[0, 0]
    assert vQ < 0
    assert np.sum(np.abs(ev) > 1e-12 * np.abs(ev).max()) == 1
    kk, cs, vs = O.basis(len(kpt), p.nc, p.nv)
    u = np.einsum("iw,iw->i", np.conj(vq[kk, cs]), vec[kk, vs])
    np.testing.assert_allclose(ev.max(), -vQ * np.vdot(u, u).real, rtol=1e-10)


def test_fermi_weights_and_gap_corrections():
    """fermidisteh: f_v - f_c = tanh(x/2) for E_v = -E_c with x = E_c/(kb T); T = 0 reads as 1e-8 K (a step);
    the gap corrections vanish as T -> 0 and are negative above."""
    kb = O.KB_F32
    for T in (50.0, 300.0, 3000.0):
        ec = np.array([0.01, 0.1, 0.75])
        np.testing.assert_allclose(O.fermidisteh(ec, -ec, T), np.tanh(ec / (kb * T) / 2), rtol=1e-12)
    assert np.all(O.fermidisteh(np.array([0.5, 2.0]), np.array([-0.5, -1.0]), 0.0) == 1.0)
    assert O.fermidisteh(np.array([0.3]), np.array([0.2]), 0.0)[0] == 0.0   # both empty
    assert abs(O.gapcortemp(2.0, 0.02, 1e-3)) < 1e-12 and O.gapcortemp(2.0, 0.02, 300.0) < 0
    assert abs(O.gapcortemp2(0.1, 300.0, 1.0)) < 1e-12 and O.gapcortemp2(0.1, 300.0, 600.0) < 0


def test_temperature_bse_reduces_to_full_spectrum_at_low_temperature(small):
    """f = 1 for every transition of a 1.5 eV gap at 10 K: the temperature matrix is the plain BSE matrix and
    its eigenvalues its full spectrum; the activities sum to sum_j f_j |h_j|^2 (completeness of A)."""
    sysm, p, kpt, eigv, vec, nocp = small
    r = O.bsesolvertemp(sysm, p, 10.0)
    assert np.all(r["fdeh"] == 1.0)
    H = O.bse_build(eigv, vec, kpt, p, sysm.rlat)
    np.testing.assert_allclose(r["Ws"], np.linalg.eigvalsh(H), atol=1e-11)
    hx = O.optsp_all(eigv, vec, kpt, sysm, p)[0]
    # sum_n s_n conj(t_n) = h^T A A^H conj(h f) = h^T conj(h f) (A unitary)
    np.testing.assert_allclose(r["acts"]["xx"].sum(), np.sum(np.abs(hx) ** 2 * r["fdeh"]), rtol=1e-10)
    hot = O.bsesolvertemp(sysm, p, 4000.0, ta="BE", st=0.05, phavg=300.0)
    assert hot["tcor"] < 0 and np.all(hot["fdeh"] < 1.0)
    np.testing.assert_allclose(hot["E"], np.conj(hot["E"].T), atol=1e-15)


@pytest.mark.parametrize("name", ["hex8_6x6", "hex8_24x24"])
def test_golden_fixtures(name):
    from tests.golden.make_golden import input_digest

    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    sysm, p = S.workload(name)
    assert str(g["digest"]) == input_digest(sysm), "the seeded input generator changed"
    r = O.bsesolver(sysm, p)
    np.testing.assert_allclose(r["E"], g["E"], atol=1e-11)
    np.testing.assert_allclose(r["eigv"], g["eigv"], atol=1e-12)
    spec = O.bsedielraw(r["Ws"], r["acts"], p.ngrid, sysm.rlat, p)
    for c in ("xx", "yy", "zz"):
        np.testing.assert_allclose(spec[c], g["spec_" + c], rtol=1e-8, atol=1e-10)


def test_next_rows_golden_fixture():
    """The oracle's finite-Q, temperature, IPA-record and BZ-activity outputs on the small case against the
    committed fixture (tests/golden/hex8_6x6_next_rows.npz)."""
    from tests.golden.make_golden import input_digest

    g = np.load(os.path.join(HERE, "golden", "hex8_6x6_next_rows.npz"))
    sysm, p = S.workload("hex8_6x6")
    assert str(g["digest"]) == input_digest(sysm), "the seeded input generator changed"
    qpath = O.kpathbse(sysm.rlat, np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]]), 3)
    np.testing.assert_array_equal(qpath, g["qpath"])
    np.testing.assert_allclose(O.bsebnds(sysm, p, qpath), g["exk"], atol=1e-11)
    np.testing.assert_allclose(O.bsebndstemp(sysm, p, qpath, 3000.0, "BE", 0.05, 300.0), g["exk_temp"], atol=1e-11)
    r = O.bsesolvertemp(sysm, p, 4000.0, "VE", 2.0e-4, 0.02)
    np.testing.assert_allclose(r["Ws"], g["W_4000"], atol=1e-11)
    np.testing.assert_allclose(r["fdeh"], g["fdeh_4000"], atol=1e-14)
    for c in ("xx", "yy", "zz", "sp", "sm"):
        np.testing.assert_allclose(r["acts"][c].sum(), g[f"actsum_{c}_4000"], rtol=1e-10)
    np.testing.assert_allclose(O.spoptpolbz(sysm, p), g["bz_act"], rtol=1e-10, atol=1e-13)


def test_c_restatement_matches_numpy(built, small):
    """The element-by-element C loop (the timed CPU baseline) equals the vectorised oracle."""
    import __graft_entry__ as g

    sysm, p, kpt, eigv, vec, _ = small
    lib = ctypes.CDLL(g.ORACLE_SO)

    class Coul(ctypes.Structure):
        _fields_ = [("coultype", ctypes.c_int), ("ngrid", ctypes.c_int * 3), ("ktol", ctypes.c_double),
                    ("ediel", ctypes.c_double * 3), ("ez", ctypes.c_double), ("w", ctypes.c_double),
                    ("r0", ctypes.c_double), ("lc", ctypes.c_double), ("rlat", ctypes.c_double * 9)]

    cp = Coul()
    cp.coultype = 6
    for i in range(3):
        cp.ngrid[i] = p.ngrid[i]
        cp.ediel[i] = p.ediel[i]
    cp.ktol, cp.ez, cp.w, cp.r0, cp.lc = p.ktol, p.ez, p.w_coul, p.r0, p.lc
    for i in range(9):
        cp.rlat[i] = sysm.rlat.reshape(-1)[i]
    dim = p.dim
    out = np.zeros((dim, dim), dtype=np.complex128)
    e, v, k = np.ascontiguousarray(eigv), np.ascontiguousarray(vec), np.ascontiguousarray(kpt)
    lib.oracle_build_rows(len(kpt), p.nc, p.nv, sysm.w90basis, e.ctypes.data_as(ctypes.c_void_p),
                          v.ctypes.data_as(ctypes.c_void_p), k.ctypes.data_as(ctypes.c_void_p), ctypes.byref(cp),
                          ctypes.c_long(0), ctypes.c_long(dim), out.ctypes.data_as(ctypes.c_void_p))
    H = O.bse_build(eigv, vec, kpt, p, sysm.rlat)
    iu = np.triu_indices(dim)
    np.testing.assert_allclose(out[iu], H[iu], rtol=0, atol=1e-14)


@pytest.mark.parametrize("name", ["hex12_60x60", "cubic16_16x16x16"])
def test_fullsize_fixture_consistent(name):
    """The full-size oracle fixtures: the stored system is the seeded one, the stored ARPACK residuals are
    below 1e-8 eV, and the stored spectra are bsedielraw of the stored energies and activities."""
    import os

    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", name + "_oracle.npz")
    g = np.load(path)
    sysm = S.system_from_arrays(g)
    regen, p = S.workload(name)
    np.testing.assert_allclose(sysm.hop, regen.hop, rtol=0, atol=1e-12)
    np.testing.assert_allclose(sysm.ihop, regen.ihop, rtol=0, atol=1e-12)
    np.testing.assert_array_equal(sysm.rvec, regen.rvec)
    assert abs(sysm.efermi - regen.efermi) < 1e-12
    assert g["E"].shape == (p.nev,) and np.all(np.diff(g["E"]) > 0)
    assert np.all(g["residual"] < 1e-8)
    Ws = np.zeros(p.dim)
    Ws[: p.nev] = g["E"]
    acts = {c: np.concatenate([g["act_" + c], np.zeros(p.dim - p.nev)]) for c in O.COMPONENTS}
    spec = O.bsedielraw(Ws, acts, p.ngrid, sysm.rlat, p)
    for c in ("xx", "yy", "zz"):
        np.testing.assert_allclose(spec[c], g["spec_" + c], rtol=1e-12, atol=1e-14)
