"""Finite-Q BSE (bsebnds / matrizelbsekq) and the dense Hermitian eigenvalue solver that replaces its ZHEEV
calls, through the C ABI against the oracle.

Tolerances: dense eigenvalues 1e-12 of the matrix norm (FP64 Householder + bisection are backward stable);
finite-Q matrix 1e-12 relative to its largest element; finite-Q exciton energies 1e-9 eV."""
import numpy as np
import pytest

from oracle import wtb_oracle as O
from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _herm(n, rng, spectrum=None):
    X = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    if spectrum is None:
        return (X + X.conj().T) / 2
    Q, _ = np.linalg.qr(X)
    return (Q * spectrum) @ Q.conj().T


@pytest.mark.parametrize("n", [1, 2, 3, 17, 64, 129, 300, 777])
def test_zheev_random(ctx, n):
    rng = np.random.default_rng(n)
    A = _herm(n, rng)
    W = ctx.zheev(A)
    ref = np.linalg.eigvalsh(A)
    assert np.all(np.diff(W) >= 0)
    assert np.max(np.abs(W - ref)) <= 1e-12 * max(1.0, np.abs(ref).max()) * max(1.0, np.sqrt(n)), \
        np.max(np.abs(W - ref))


def test_zheev_edge_cases(ctx):
    rng = np.random.default_rng(5)
    # diagonal: every reflector is the identity (tau = 0)
    d = rng.standard_normal(50)
    np.testing.assert_allclose(ctx.zheev(np.diag(d).astype(np.complex128)), np.sort(d), atol=1e-14)
    # zero matrix: the bisection bracket closes on zero to within the pivot guard (~1e-307)
    np.testing.assert_allclose(ctx.zheev(np.zeros((9, 9), dtype=np.complex128)), np.zeros(9), atol=1e-300)
    # clusters of equal eigenvalues
    spec = np.repeat([-1.0, 0.5, 2.0, 2.0 + 1e-13], [5, 7, 4, 4])
    A = _herm(20, rng, spec)
    np.testing.assert_allclose(ctx.zheev(A), np.sort(spec), atol=1e-12)
    # only the upper triangle is read (ZHEEV 'U'): garbage below the diagonal and imaginary diagonal parts
    B = _herm(40, rng)
    G = np.triu(B) + np.tril(rng.standard_normal((40, 40)) * 1e3, -1) + 1j * np.diag(rng.standard_normal(40))
    np.testing.assert_allclose(ctx.zheev(G), np.linalg.eigvalsh(B), atol=1e-12 * np.abs(B).max() * 10)
    # large dynamic range
    spec = np.concatenate([np.linspace(1e-6, 1e-3, 10), np.linspace(10.0, 20.0, 10)])
    A = _herm(20, rng, spec)
    np.testing.assert_allclose(ctx.zheev(A), np.sort(spec), atol=1e-13 * 20)


@pytest.fixture(scope="module")
def small_bands():
    sysm, p = S.workload("hex8_6x6")
    kpt = O.monhkhorst_pack(*p.ngrid, p.mshift, sysm.rlat)
    eigv, vec, nocp = O.bands(sysm, p, kpt)
    return sysm, p, kpt, eigv, vec


@pytest.mark.parametrize("q", [(0.0, 0.0, 0.0, 0.0), (0.3, 0.05, 0.02, 0.0), (0.7, -0.2, 0.1, 0.0)])
def test_bse_build_q(ctx, small_bands, q):
    sysm, p, kpt, eigv, vec = small_bands
    ctx.set_hr(sysm)
    q = np.array(q)
    kq = O.monhkhorst_packq(q, *p.ngrid, p.mshift, sysm.rlat)
    eq, vq, _ = O.bands(sysm, p, kq)
    ref = O.bse_build_q(eigv, vec, eq, vq, kpt, q, p, sysm.rlat)
    H = ctx.bse_build_q(p, q)
    # the band vectors carry a gauge (phase) per (k, band): compare gauge-invariant quantities
    np.testing.assert_allclose(np.diag(H).real, np.diag(ref).real, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(np.abs(H), np.abs(ref), atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(np.linalg.eigvalsh(H), np.linalg.eigvalsh(ref), atol=1e-11 * np.abs(ref).max())


def test_bsebnds_small(ctx, small_bands, tmp_path):
    """The whole Q loop on a path through Gamma (Q = 0: no exchange) against the oracle's ZHEEV spectrum, and
    its bands_bse.dat read back."""
    sysm, p, kpt, eigv, vec = small_bands
    ctx.set_hr(sysm)
    ks = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.5, 0.0, 0.0], [1 / 3, 1 / 3, 0.0]])
    qpath = O.kpathbse(sysm.rlat, ks, 3)
    exk = ctx.bsebnds(p, qpath)
    ref = O.bsebnds(sysm, p, qpath)
    assert exk.shape == ref.shape == (p.dim, len(qpath))
    assert np.max(np.abs(exk - ref)) <= 1e-9, np.max(np.abs(exk - ref))
    # Q = 0 reproduces the plain BSE spectrum
    H0 = O.bse_build(eigv, vec, kpt, p, sysm.rlat)
    np.testing.assert_allclose(exk[:, 0], np.linalg.eigvalsh(H0), atol=1e-9)
    from wtb_gb300 import api
    path = str(tmp_path / "bands_bse.dat")
    api.write_bands_bse(path, qpath, exk)
    lines = open(path).read().splitlines()
    assert len(lines) == p.dim * (len(qpath) + 1)
    assert lines[len(qpath)] == "" and lines[1] == O.list_directed_record([("r4", qpath[1, 0]), ("r8", exk[0, 1])])
    back = np.array([[float(t) for t in ln.split()] for ln in lines if ln])
    assert np.array_equal(back[:, 1], exk.reshape(-1))          # band-major, every REAL(8) energy exactly
    assert np.array_equal(back[: len(qpath), 0].astype(np.float32), qpath[:, 0].astype(np.float32))


def test_bsebnds_2304(ctx):
    """dim 2304 (24 x 24 mesh, 2v2c), one Q: the GPU spectrum against LAPACK on the oracle's matrix."""
    sysm, p = S.workload("hex8_24x24")
    ctx.set_hr(sysm)
    q = np.array([0.2, 0.04, 0.0, 0.0])
    exk = ctx.bsebnds(p, q.reshape(1, 4))[:, 0]
    kpt = O.monhkhorst_pack(*p.ngrid, p.mshift, sysm.rlat)
    eigv, vec, _ = O.bands(sysm, p, kpt)
    kq = O.monhkhorst_packq(q, *p.ngrid, p.mshift, sysm.rlat)
    eq, vq, _ = O.bands(sysm, p, kq)
    ref = np.linalg.eigvalsh(O.bse_build_q(eigv, vec, eq, vq, kpt, q, p, sysm.rlat))
    assert np.max(np.abs(exk - ref)) <= 1e-9, np.max(np.abs(exk - ref))


@pytest.mark.parametrize("n", [1, 2, 5, 64, 300, 700])
def test_zheev_vectors_random(ctx, n):
    """ZHEEV('V'): eigenvalues as LAPACK's, residual and orthonormality at FP64 level."""
    rng = np.random.default_rng(100 + n)
    A = _herm(n, rng)
    W, Z = ctx.zheev_vectors(A)
    nrm = max(1.0, np.abs(np.linalg.eigvalsh(A)).max())
    np.testing.assert_allclose(W, np.linalg.eigvalsh(A), atol=1e-12 * nrm * np.sqrt(n))
    assert np.abs(A @ Z - Z * W).max() <= 1e-11 * nrm, np.abs(A @ Z - Z * W).max()
    assert np.abs(Z.conj().T @ Z - np.eye(n)).max() <= 1e-10


def test_zheev_vectors_degenerate_and_diagonal(ctx):
    rng = np.random.default_rng(9)
    spec = np.repeat([-2.0, 0.3, 0.3 + 1e-12, 1.0, 4.0], [6, 5, 3, 1, 9])
    A = _herm(len(spec), rng, spec)
    W, Z = ctx.zheev_vectors(A)
    np.testing.assert_allclose(W, np.sort(spec), atol=1e-12)
    assert np.abs(A @ Z - Z * W).max() <= 1e-11
    assert np.abs(Z.conj().T @ Z - np.eye(len(spec))).max() <= 1e-10
    D = np.diag(rng.standard_normal(30)).astype(np.complex128)
    D[5, 5] = D[7, 7] = D[11, 11]
    W, Z = ctx.zheev_vectors(D)
    assert np.abs(D @ Z - Z * W).max() <= 1e-13
    assert np.abs(Z.conj().T @ Z - np.eye(30)).max() <= 1e-12


def _cluster_sums(W, x, tol=1e-7):
    """sums of x over groups of (near-)equal W: the gauge-invariant content of per-exciton activities"""
    out, cur, last = [], 0.0, None
    for w, v in zip(W, x):
        if last is not None and w - last >= tol:
            out.append(cur)
            cur = 0.0
        cur += v
        last = w
    out.append(cur)
    return np.array(out)


@pytest.mark.parametrize("temp,ta,st,phavg", [(300.0, "FA", 0.0, 0.0), (4000.0, "VE", 2.0e-4, 0.02),
                                              (4000.0, "BE", 0.05, 300.0), (0.0, "FA", 0.0, 0.0)])
def test_bsesolvertemp_small(ctx, small_bands, temp, ta, st, phavg):
    """bsesolvertemp against the oracle: every eigenvalue 1e-9 eV, f 1e-12, activities summed over
    degenerate groups 1e-8 of the largest, the broadened spectra 1e-8, and the eigenvectors of the weighted
    matrix (residual, orthonormality)."""
    sysm, p, kpt, eigv, vec = small_bands
    ctx.set_hr(sysm)
    out = ctx.bsesolvertemp(p, temp, ta, st, phavg, want_vectors=True)
    ref = O.bsesolvertemp(sysm, p, temp, ta, st, phavg)
    np.testing.assert_allclose(out["Ws"], ref["Ws"], atol=1e-9)
    np.testing.assert_allclose(out["fdeh"], ref["fdeh"], atol=1e-12)
    for c in O.COMPONENTS + ("sp", "sm"):
        a, b = _cluster_sums(ref["Ws"], out["acts"][c]), _cluster_sums(ref["Ws"], ref["acts"][c])
        np.testing.assert_allclose(a, b, atol=1e-8 * max(1.0, np.abs(b).max()))
    spec = O.bsedielraw(out["Ws"], out["acts"], p.ngrid, sysm.rlat, p)
    spec_ref = O.bsedielraw(ref["Ws"], ref["acts"], p.ngrid, sysm.rlat, p)
    for c in ("xx", "yy", "zz"):
        np.testing.assert_allclose(spec[c], spec_ref[c], rtol=1e-8, atol=1e-10)
    # the eigenvectors against the weighted matrix in the library's own band gauge (the oracle's bands may
    # differ by signs, which change no output above): the direct matrix of the same bands, weighted as
    # ZHEEV 'U' reads matrizelbsetemp
    HE = out["HE"]
    D = ctx.bse_build(p)
    f = out["fdeh"]
    idx = np.arange(p.dim)
    E = D * f[np.minimum(idx[:, None], idx[None, :])]
    Vkk = np.diag(O.coulomb_table(kpt, kpt, p, sysm.rlat))[idx // (p.nc * p.nv)]
    E[idx, idx] = D[idx, idx] + Vkk * (f - 1.0)
    assert np.abs(E @ HE - HE * out["Ws"]).max() <= 1e-10
    assert np.abs(HE.conj().T @ HE - np.eye(p.dim)).max() <= 1e-10


def test_bsesolvertemp_2304(ctx):
    """dim 2304 (24 x 24 mesh, 2v2c) at 600 K: every exciton energy 1e-9 eV and the broadened spectra 1e-8
    against the oracle's dense eigendecomposition."""
    sysm, p = S.workload("hex8_24x24")
    ctx.set_hr(sysm)
    out = ctx.bsesolvertemp(p, 600.0, "VE", 3.0e-4, 0.03)
    ref = O.bsesolvertemp(sysm, p, 600.0, "VE", 3.0e-4, 0.03)
    np.testing.assert_allclose(out["Ws"], ref["Ws"], atol=1e-9)
    spec = O.bsedielraw(out["Ws"], out["acts"], p.ngrid, sysm.rlat, p)
    spec_ref = O.bsedielraw(ref["Ws"], ref["acts"], p.ngrid, sysm.rlat, p)
    for c in ("xx", "yy", "zz", "xy"):
        np.testing.assert_allclose(spec[c], spec_ref[c], rtol=1e-8, atol=1e-9 * np.abs(spec_ref[c]).max())


@pytest.mark.parametrize("temp,ta,st,phavg", [(300.0, "FA", 0.0, 0.0), (3000.0, "BE", 0.05, 300.0)])
def test_bsebndstemp_small(ctx, small_bands, temp, ta, st, phavg):
    """bsebndstemp: the finite-Q Q loop with the temperature weighting and gap correction, against the oracle."""
    sysm, p, kpt, eigv, vec = small_bands
    ctx.set_hr(sysm)
    ks = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])
    qpath = O.kpathbse(sysm.rlat, ks, 3)
    exk = ctx.bsebndstemp(p, qpath, temp, ta, st, phavg)
    ref = O.bsebndstemp(sysm, p, qpath, temp, ta, st, phavg)
    assert np.max(np.abs(exk - ref)) <= 1e-9, np.max(np.abs(exk - ref))
    if temp < 1000:   # f = 1 for a 1.5 eV gap: the plain finite-Q spectrum
        np.testing.assert_allclose(exk, O.bsebnds(sysm, p, qpath), atol=1e-9)


def test_spoptics_temp(ctx, small_bands):
    """bsesolvertemp's IPA records: bands with scs + tcor, activity columns weighted by f_v - f_c."""
    sysm, p, kpt, eigv, vec = small_bands
    import dataclasses
    ctx.set_hr(sysm)
    temp, st, phavg = 3000.0, 0.05, 300.0
    rec = ctx.spoptics_temp(p, temp, "BE", st, phavg)
    s2 = dataclasses.replace(sysm, scs=sysm.scs + O.gapcortemp2(st, phavg, temp))
    e2, v2, nocp = O.bands(s2, p, kpt)
    hr = O.optsp_all(e2, v2, kpt, s2, p)
    kk, cs, vs = O.basis(len(kpt), p.nc, p.nv)
    f = O.fermidisteh(e2[kk, cs], e2[kk, vs], temp)
    assert np.all(f < 1.0)
    ref = O.spoptics_records(e2, kpt, nocp, hr, p.nv, p.nc, f)
    assert np.all(np.diff(rec[:, 6]) >= 0)
    np.testing.assert_allclose(rec[:, 6], ref[:, 6], rtol=2e-7, atol=1e-6)
    amax = np.abs(ref[:, 7:15]).max()
    # rows matched by (k-point, c, v)
    key = lambda r: (round(float(r[0]), 4), round(float(r[1]), 4), round(float(r[2]), 4), int(r[4]), int(r[5]))
    a = {key(r): r for r in rec}
    for r in ref:
        np.testing.assert_allclose(a[key(r)][7:15], r[7:15], rtol=0, atol=1e-6 * amax)


def test_bse_q_eigenpairs(ctx, small_bands):
    """bsebnds with bsewf: eigenvalues as wtb_bsebnds, the selected eigenvectors satisfy H_Q z = w z for the
    finite-Q matrix of the same bands, orthonormal."""
    sysm, p, kpt, eigv, vec = small_bands
    ctx.set_hr(sysm)
    q = np.array([0.3, 0.05, 0.02, 0.0])
    W, Z = ctx.bse_q_eigenpairs(p, q, il=2, nvec=5)
    np.testing.assert_allclose(W, ctx.bsebnds(p, q.reshape(1, 4))[:, 0], atol=1e-12)
    H = ctx.bse_build_q(p, q)
    assert np.abs(H @ Z - Z * W[1:6]).max() <= 1e-11
    assert np.abs(Z.conj().T @ Z - np.eye(5)).max() <= 1e-11


def test_next_rows_argument_errors(ctx, small_bands):
    """bad arguments of the full-spectrum entry points come back as WTB_EBADARG with a message, not a fault"""
    from wtb_gb300 import api

    sysm, p, kpt, eigv, vec = small_bands
    ctx.set_hr(sysm)
    with pytest.raises(api.WTBError) as e:
        ctx.bsesolvertemp(p, 300.0, ta=5)
    assert e.value.code == api.WTB_EBADARG and "temperature" in str(e.value)
    with pytest.raises(api.WTBError) as e:
        ctx.bsesolvertemp(p, -1.0)
    assert e.value.code == api.WTB_EBADARG
    with pytest.raises(api.WTBError) as e:
        ctx.bsebnds(p, np.zeros((0, 4)))
    assert e.value.code == api.WTB_EBADARG
    big = S.BSEParams(**{**p.__dict__})
    big.ngrid = (80, 80, 1)                            # dim 25,600 > 20,000: refused before any allocation
    with pytest.raises(api.WTBError) as e:
        ctx.bsebnds(big, np.zeros((1, 4)))
    assert e.value.code == api.WTB_EBADARG and "dim <= 20000" in str(e.value)
    with pytest.raises(api.WTBError):
        ctx.bse_q_eigenpairs(p, np.zeros(4), il=p.dim, nvec=2)
    with pytest.raises(api.WTBError):
        api.kpathbse(sysm.rlat[0], sysm.rlat[1], sysm.rlat[2], np.zeros((2, 3)), 1)
    # the context stays usable
    np.testing.assert_allclose(ctx.zheev(np.diag([3.0, 1.0, 2.0]).astype(complex)), [1.0, 2.0, 3.0], atol=1e-14)


def test_next_rows_against_golden_fixture(ctx):
    """The GPU's finite-Q, temperature, IPA-record and BZ-activity outputs against the committed fixture made
    by the oracle (tests/golden/hex8_6x6_next_rows.npz)."""
    import os

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hex8_6x6_next_rows.npz"))
    sysm, p = S.workload("hex8_6x6")
    ctx.set_hr(sysm)
    np.testing.assert_allclose(ctx.bsebnds(p, g["qpath"]), g["exk"], atol=1e-9)
    np.testing.assert_allclose(ctx.bsebndstemp(p, g["qpath"], 3000.0, "BE", 0.05, 300.0), g["exk_temp"], atol=1e-9)
    for T, ta, st, ph in ((300.0, "FA", 0.0, 0.0), (4000.0, "VE", 2.0e-4, 0.02)):
        out = ctx.bsesolvertemp(p, T, ta, st, ph)
        np.testing.assert_allclose(out["Ws"], g[f"W_{int(T)}"], atol=1e-9)
        np.testing.assert_allclose(out["fdeh"], g[f"fdeh_{int(T)}"], atol=1e-12)
        for c in ("xx", "yy", "zz", "sp", "sm"):
            ref = float(g[f"actsum_{c}_{int(T)}"])
            assert abs(out["acts"][c].sum() - ref) <= 1e-8 * max(1.0, abs(ref)), (T, c)
    rec = ctx.spoptics(p)
    np.testing.assert_allclose(rec[:, 6], g["sp_records"][:, 6], rtol=2e-7, atol=1e-6)
    np.testing.assert_allclose(ctx.spoptpolbz(p), g["bz_act"], rtol=1e-9, atol=1e-12 * np.abs(g["bz_act"]).max())
