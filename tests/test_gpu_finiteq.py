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


def test_bsebnds_small(ctx, small_bands):
    """The whole Q loop on a path through Gamma (Q = 0: no exchange) against the oracle's ZHEEV spectrum."""
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
