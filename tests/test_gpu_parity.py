"""Parity of the CUDA path (through the C ABI) against the FP64 oracle on seeded systems.

Tolerances: integer outputs exact; per-k band energies 1e-11 eV; band vectors 1e-9 (after the
first-component-real gauge, sign included); V table and FP64 dense build 1e-12 relative; FP32 build
2e-6 of the largest element; exciton energies 1e-5 eV (the acceptance bound) in every precision mode;
spectra 1e-4 relative L2.
"""
import numpy as np
import pytest

from oracle import wtb_oracle as O
from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MODES = [("fp64", "dense"), ("fp32", "dense"), ("fp64", "matfree"), ("fp32", "matfree"), ("bf16x3", "matfree"),
         ("bf16x6", "matfree")]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def small():
    sysm, p = S.workload("hex8_6x6")
    ref = O.bsesolver(sysm, p, with_vectors=True)
    return sysm, p, ref


@pytest.fixture(scope="module")
def c1():
    sysm, p = S.workload("hex8_24x24")
    ref = O.bsesolver(sysm, p, with_vectors=False)
    return sysm, p, ref


def test_bands_match_zheev(ctx, small):
    sysm, p, ref = small
    ctx.set_hr(sysm)
    eigv, vec, nocp = ctx.eigsys_mesh(ref["kpt"], p.nv, p.nc)
    np.testing.assert_array_equal(nocp, ref["nocpk"])
    np.testing.assert_allclose(eigv, ref["eigv"], rtol=0, atol=1e-11)
    np.testing.assert_allclose(vec, O.gauge_fix(ref["vec"]), rtol=0, atol=1e-9)
    # ZHEEV('L') leaves the first component real: the oracle's vectors equal ours up to a sign
    assert np.max(np.abs(ref["vec"][..., 0].imag)) < 1e-12


def test_eigsys_reference_argument_list(built, small):
    from wtb_gb300 import api

    sysm, p, ref = small
    k = ref["kpt"][7]
    nocp, e, av = api.eigsys(1, sysm.scs, 0.0, 0, sysm.ffactor, k[0], k[1], k[2], sysm.w90basis, sysm.nvec,
                             sysm.rlat, sysm.rvec, sysm.hop, sysm.ihop, sysm.efermi)
    e_ref, av_ref, nocp_ref = O.eigsys(k, sysm)
    assert nocp == nocp_ref
    np.testing.assert_allclose(e, e_ref, atol=1e-11)
    np.testing.assert_allclose(av, O.gauge_fix(av_ref), atol=1e-9)


def test_scissor_shift(ctx, small):
    sysm, p, ref = small
    s2 = sysm.copy()
    s2.scs = 0.37
    ctx.set_hr(s2)
    eigv, _, _ = ctx.eigsys_mesh(ref["kpt"], p.nv, p.nc)
    e_ref, _, nocp = O.eigsys(ref["kpt"][3], s2)
    np.testing.assert_allclose(eigv[3], e_ref[nocp - p.nv: nocp + p.nc], atol=1e-11)
    ctx.set_hr(sysm)


@pytest.mark.parametrize("coultype", ["V2DRK", "V3DL", "V3D", "V2DK", "V2DOH", "V2DT", "V2DT2", "V0DT", "V1DT"])
def test_coulomb_table(ctx, small, coultype):
    sysm, p, ref = small
    ctx.set_hr(sysm)
    q = S.BSEParams(**{**p.__dict__})
    q.coultype = coultype
    q.ediel = (1.5, 4.0, 2.0)
    q.ez, q.w_coul, q.r0, q.lc = 2.0, 0.7, 35.0, 6.0
    kpt = ref["kpt"]
    V = ctx.coulomb_table(q, kpt)
    Vref = O.coulomb_table(kpt, kpt, q, sysm.rlat)
    np.testing.assert_allclose(V, Vref, rtol=1e-12, atol=1e-14 * np.abs(Vref).max())


def test_optics_matrix_elements(ctx, small):
    sysm, p, ref = small
    ctx.set_hr(sysm)
    ctx.eigsys_mesh(ref["kpt"], p.nv, p.nc)
    hr = ctx.optsp(p)
    h_ref = np.stack(O.optsp_all(ref["eigv"], O.gauge_fix(ref["vec"]), ref["kpt"], sysm, p))
    np.testing.assert_allclose(hr, h_ref, rtol=0, atol=1e-10 * np.abs(h_ref).max())


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 2e-6)])
def test_dense_build(ctx, small, precision, tol):
    sysm, p, ref = small
    ctx.set_hr(sysm)
    ctx.eigsys_mesh(ref["kpt"], p.nv, p.nc)
    H = ctx.bse_build(p, precision=precision)
    Href = O.bse_build(ref["eigv"], O.gauge_fix(ref["vec"]), ref["kpt"], p, sysm.rlat)
    assert np.abs(H - H.conj().T).max() <= tol * np.abs(Href).max()
    np.testing.assert_allclose(H, Href, rtol=0, atol=tol * np.abs(Href).max())


MATVEC_TOL = {("fp64", "dense"): 1e-13, ("fp32", "dense"): 2e-6, ("fp64", "matfree"): 1e-13,
              ("fp32", "matfree"): 2e-6, ("bf16x3", "matfree"): 2e-4, ("bf16x6", "matfree"): 2e-6}


@pytest.mark.parametrize("precision,op", MODES)
@pytest.mark.parametrize("ncol", [1, 5, 16, 20])
def test_operator_matvec(ctx, small, precision, op, ncol):
    """Every operator variant against the oracle's dense FP64 matrix, relative to ||H x||."""
    sysm, p, ref = small
    ctx.set_hr(sysm)
    ctx.eigsys_mesh(ref["kpt"], p.nv, p.nc)
    Href = O.bse_build(ref["eigv"], O.gauge_fix(ref["vec"]), ref["kpt"], p, sysm.rlat)
    rng = np.random.default_rng(ncol)
    X = rng.normal(size=(p.dim, ncol)) + 1j * rng.normal(size=(p.dim, ncol))
    Y = ctx.bse_matvec(p, X, precision=precision, op=op)
    Yref = Href @ X
    err = np.linalg.norm(Y - Yref, axis=0) / np.linalg.norm(Yref, axis=0)
    assert err.max() <= MATVEC_TOL[(precision, op)], err


@pytest.mark.parametrize("name,P", [("hex8_6x6", 32), ("hex8_24x24", 64)])
def test_fft_operator_on_the_mesh(ctx, name, P):
    """On a Monkhorst-Pack mesh (bands of the mesh itself, not a k-point list) the FP32 matrix-free operator is the
    FFT convolution of the Coulomb stencil (transform size P): against the oracle's FP64 factored operator,
    relative to ||H x|| (the bound of the CUDA-core FP32 product)."""
    sysm, p = S.workload(name)
    ctx.set_hr(sysm)
    ctx.bsesolver(p, precision="fp64", op="matfree")  # stages the mesh and its bands
    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, _ = O.bands(sysm, p, kpt)
    rng = np.random.default_rng(P)
    X = rng.normal(size=(p.dim, 20)) + 1j * rng.normal(size=(p.dim, 20))
    Y = ctx.bse_matvec(p, X, precision="fp32", op="matfree")
    assert ctx.operator_form() == "FP32 FFT convolution"
    Yref = O.bse_matvec_factored(X, eigv, O.gauge_fix(vec), kpt, p, sysm.rlat)
    err = np.linalg.norm(Y - Yref, axis=0) / np.linalg.norm(Yref, axis=0)
    assert err.max() <= 2e-6, err


def test_slepc_solver_dense(ctx, small):
    sysm, p, ref = small
    Href = O.bse_build(ref["eigv"], ref["vec"], ref["kpt"], p, sysm.rlat)
    EX, HE = ctx.slepc_solver(Href, 6)
    w = np.linalg.eigvalsh(Href)[:6]
    np.testing.assert_allclose(EX, w, atol=1e-9)
    R = Href @ HE - HE * EX[None, :]
    assert np.linalg.norm(R, axis=0).max() < 1e-7 * np.abs(EX).max()


@pytest.mark.parametrize("precision,op", MODES)
def test_bsesolver_small(ctx, small, precision, op):
    sysm, p, ref = small
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision=precision, op=op)
    np.testing.assert_allclose(out["E"], ref["E"], rtol=0, atol=1e-5)
    assert np.all(out["Ws"][p.nev:] == 0.0)
    dim = p.dim
    for c in ("xx", "yy", "zz"):
        assert np.all(out["acts"][c][p.nev:] == 0.0)


@pytest.mark.parametrize("precision,op", MODES)
def test_bsesolver_hex8_24x24(ctx, c1, precision, op):
    """dim 2304, 10 excitons: energies within 1e-5 eV and the spectrum within 1e-4 relative L2."""
    sysm, p, ref = c1
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision=precision, op=op)
    err = np.abs(out["E"] - ref["E"])
    assert err.max() <= 1e-5, err
    spec = O.bsedielraw(out["Ws"], out["acts"], p.ngrid, sysm.rlat, p)
    spec_ref = O.bsedielraw(ref["Ws"], ref["acts"], p.ngrid, sysm.rlat, p)
    for c in ("xx", "yy", "zz"):
        assert rel_l2(spec[c][:, 2], spec_ref[c][:, 2]) <= 1e-4, c


def test_spectrum_kernel(ctx, c1, tmp_path):
    """bsedielraw's spectra against the oracle, and bse_diel_xx.dat written from them and read back as
    bseoptprop reads it (energies exactly, eps1 and eps2 at single precision)."""
    sysm, p, ref = c1
    ctx.set_hr(sysm)
    d = ctx.bsedielraw(p, ref["Ws"], ref["acts"])
    d_ref = O.bsedielraw(ref["Ws"], ref["acts"], p.ngrid, sysm.rlat, p)
    for c in O.COMPONENTS:
        np.testing.assert_allclose(d[c], d_ref[c], rtol=1e-10, atol=1e-12 * max(1.0, np.abs(d_ref[c]).max()))
    from wtb_gb300 import api
    path = str(tmp_path / "bse_diel_xx.dat")
    api.write_diel(path, d["xx"])
    lines = open(path).read().splitlines()
    back = np.array([[float(t) for t in ln.split()] for ln in lines[1:]])
    assert lines[0] == " #  energy  real  imag" and back.shape == d["xx"].shape
    assert np.array_equal(back[:, 0], d["xx"][:, 0])
    assert np.array_equal(back[:, 1:].astype(np.float32), d["xx"][:, 1:].astype(np.float32))


def test_optprops_kernel(ctx, c1):
    sysm, p, ref = c1
    ctx.set_hr(sysm)
    d_ref = O.bsedielraw(ref["Ws"], ref["acts"], p.ngrid, sysm.rlat, p)
    props = ctx.bseoptprop(d_ref)
    for c in O.COMPONENTS:
        om, e1, e2 = d_ref[c][:, 0], d_ref[c][:, 1], d_ref[c][:, 2]
        pr = O.optprops(e1, e2, om)
        for nm in ("refr", "ext", "refl", "abs", "eloss"):
            np.testing.assert_allclose(props[nm][c], pr[nm], rtol=1e-9, atol=1e-12)


def test_spectrum_pol_kernel(ctx, c1):
    """bsedielrawpol: xx yy zz sp sm all with rtype 1."""
    sysm, p, ref = c1
    ctx.set_hr(sysm)
    d = ctx.bsedielrawpol(p, ref["Ws"], ref["acts"])
    d_ref = O.bsedielrawpol(ref["Ws"], ref["acts"], p.ngrid, sysm.rlat, p)
    for c in O.POL_COMPONENTS:
        np.testing.assert_allclose(d[c], d_ref[c], rtol=1e-10, atol=1e-12 * max(1.0, np.abs(d_ref[c]).max()))
    props = ctx.bseoptproppol(d_ref)
    for c in O.POL_COMPONENTS:
        om, e1, e2 = d_ref[c][:, 0], d_ref[c][:, 1], d_ref[c][:, 2]
        pr = O.optprops(e1, e2, om)
        for nm in ("refr", "ext", "refl", "abs", "eloss"):
            np.testing.assert_allclose(props[nm][c], pr[nm], rtol=1e-9, atol=1e-12)


def _by_transition(rec):
    """rows keyed by (k-point, conduction slot, valence slot)"""
    return {(round(float(r[0]), 4), round(float(r[1]), 4), round(float(r[2]), 4), int(r[4]), int(r[5])): r
            for r in rec}


@pytest.mark.parametrize("precision,op", [("fp64", "matfree"), ("bf16x3", "matfree")])
def test_spoptics_records(ctx, small, precision, op):
    """spoptics: REAL(4) records sorted by transition energy; every (k, c, v) once; activities within the
    band solver's accuracy (FP64 bands: 1e-6 of the largest; mixed FP32/FP64 set-up: 1e-4)."""
    sysm, p, ref = small
    ctx.set_hr(sysm)
    q = S.BSEParams(**{**p.__dict__})
    q.precision, q.op = precision, op
    rec = ctx.spoptics(q)
    rr = O.spoptics_records(ref["eigv"], ref["kpt"], ref["nocpk"], ref["hr"], p.nv, p.nc)
    assert rec.dtype == np.float32 and rec.shape == rr.shape
    assert np.all(np.diff(rec[:, 6]) >= 0)
    np.testing.assert_allclose(rec[:, 6], rr[:, 6], rtol=2e-7, atol=1e-6)
    a, b = _by_transition(rec), _by_transition(rr)
    assert a.keys() == b.keys() and len(a) == p.dim
    tol = 1e-6 if precision == "fp64" else 1e-4
    amax = np.abs(rr[:, 7:15]).max(axis=0)
    for key, y in b.items():
        x = a[key]
        np.testing.assert_array_equal(x[3:6], y[3:6])
        np.testing.assert_allclose(x[7:15], y[7:15], rtol=0, atol=tol * amax.max())


def test_spdielraw_kernels(ctx, small):
    """spdielraw / spdielrawpol over the IPA transitions (every row carries activity)."""
    sysm, p, ref = small
    ctx.set_hr(sysm)
    rr = O.spoptics_records(ref["eigv"], ref["kpt"], ref["nocpk"], ref["hr"], p.nv, p.nc).astype(np.float64)
    esp = rr[:, 6]
    acts = {c: rr[:, 7 + i] for i, c in enumerate(O.COMPONENTS)}
    acts.update(sp=rr[:, 13], sm=rr[:, 14])
    for fn, ofn, comps in ((ctx.spdielraw, O.spdielraw, O.COMPONENTS),
                           (ctx.spdielrawpol, O.spdielrawpol, O.POL_COMPONENTS)):
        d = fn(p, esp, acts)
        d_ref = ofn(esp, acts, p.ngrid, sysm.rlat, p)
        for c in comps:
            np.testing.assert_allclose(d[c], d_ref[c], rtol=1e-10, atol=1e-12 * max(1.0, np.abs(d_ref[c]).max()))


def test_dielbse(ctx, small):
    sysm, p, ref = small
    A = ref["A"]
    hr = ref["hr"]
    act = ctx.dielbse(p.dim, A.shape[1], A, hr[0])
    np.testing.assert_allclose(act, O.dielbsev(A, hr[0], p.dim), rtol=1e-12, atol=1e-14)
    act = ctx.dielbse(p.dim, A.shape[1], A, hr[0], hr[1])
    np.testing.assert_allclose(act, O.dielbsep(A, hr[0], hr[1], p.dim), rtol=1e-12, atol=1e-14)


def test_error_band_window(ctx, small):
    from wtb_gb300 import api

    sysm, p, ref = small
    ctx.set_hr(sysm)
    q = S.BSEParams(**{**p.__dict__})
    q.nv = sysm.w90basis // 2 + 1
    q.nc = 1
    with pytest.raises(api.WTBError) as e:
        ctx.bsesolver(q)
    assert e.value.code == api.WTB_EBADARG
    assert "valence states higher" in str(e.value)


def test_error_arguments(ctx, small):
    from wtb_gb300 import api

    sysm, p, ref = small
    ctx.set_hr(sysm)
    q = S.BSEParams(**{**p.__dict__})
    q.ktol = 0.0
    with pytest.raises(api.WTBError) as e:
        ctx.bsesolver(q)
    assert e.value.code == api.WTB_EBADARG
    q = S.BSEParams(**{**p.__dict__})
    q.nev = p.dim + 1
    with pytest.raises(api.WTBError) as e:
        ctx.bsesolver(q)
    assert e.value.code == api.WTB_EBADARG
    bad = sysm.copy()
    bad.hop[0, 0, 0] = np.nan
    with pytest.raises(api.WTBError) as e:
        ctx.set_hr(bad)
    assert e.value.code == api.WTB_ENAN
    ctx.set_hr(sysm)


def test_determinism_fp64(ctx, small):
    sysm, p, ref = small
    ctx.set_hr(sysm)
    a = ctx.bsesolver(p, precision="fp64", op="dense", tol=1e-8)
    b = ctx.bsesolver(p, precision="fp64", op="dense", tol=1e-8)
    assert np.array_equal(a["E"], b["E"])


@pytest.mark.parametrize("sysdim", ["3D", "2D", "1D"])
def test_exciton_lifetime(ctx, small, sysdim):
    """exclft over bse_opt_diel.dat's rows (zero activity: an infinite lifetime, as the reference divides)."""
    from wtb_gb300 import api

    sysm, p, _ = small
    ctx.set_hr(sysm)
    rng = np.random.default_rng(11)
    fosc = np.zeros((40, 7))
    fosc[:, 0] = rng.uniform(1.0, 4.0, 40)
    fosc[:, 1:] = rng.uniform(0.0, 30.0, (40, 6))
    fosc[30:, 1:4] = 0.0
    lft = ctx.exciton_lifetime(sysdim, p.ngrid, fosc)
    ref = np.stack([O.exclft(sysdim, p.ngrid, sysm.rlat, fosc[:, 1] + fosc[:, 2] + fosc[:, 3], fosc[:, 0])]
                   + [O.exclft(sysdim, p.ngrid, sysm.rlat, fosc[:, c], fosc[:, 0]) for c in (1, 2, 3)], axis=1)
    np.testing.assert_allclose(lft, ref, rtol=1e-14)
    assert np.all(np.isinf(lft[30:]))
    with pytest.raises(api.WTBError) as e:
        ctx.exciton_lifetime("4D", p.ngrid, fosc)
    assert "Wrong System dimension" in str(e.value)
    # lifetimepol: the six columns of bse_opt_diel-pol.dat (energy, xx, yy, zz, sp, sm)
    fp = fosc[:, :6].copy()
    lp = ctx.exciton_lifetime(sysdim, p.ngrid, fp, pol=True)
    np.testing.assert_allclose(lp[:, :4], ref, rtol=1e-14)
    for c in (4, 5):
        np.testing.assert_allclose(lp[:, c], O.exclft(sysdim, p.ngrid, sysm.rlat, fp[:, c], fp[:, 0]), rtol=1e-14)


def test_spoptpolbz(ctx, small):
    """BZ-resolved x y z sp sm activity and dichroism per k-point against the oracle; sp + sm = 2 n^2 (x + y)
    with n = 1/sqrt(2) rounded to single precision."""
    sysm, p, _ = small
    ctx.set_hr(sysm)
    act = ctx.spoptpolbz(p)
    ref = O.spoptpolbz(sysm, p)
    np.testing.assert_allclose(act, ref, rtol=1e-9, atol=1e-12 * np.abs(ref[:, :5]).max())
    np.testing.assert_allclose(act[:, 3] + act[:, 4], 2 * O.INV_SQRT2_F32 ** 2 * (act[:, 0] + act[:, 1]), rtol=1e-12)


def test_scalar_routines_with_reference_argument_lists(built, small):
    """hlm, optsp, optdiel and the scalar potentials, one call each through their stateless entries
    (wtb_hlm, wtb_optsp_pair, wtb_optdiel, wtb_coulomb_pair), against the oracle: 1e-12 relative."""
    from wtb_gb300 import api

    sysm, p, ref = small
    kpt, eigv, vec = ref["kpt"], ref["eigv"], ref["vec"]
    for k in (0, 5, 17):
        got = api.hlm(kpt[k], sysm)
        want = O.hlm(kpt[k], sysm)
        for a in range(3):
            np.testing.assert_allclose(got[a], want[a], rtol=0, atol=1e-12 * max(1.0, np.abs(want[a]).max()))
    s32 = float(np.float32(p.cshift))
    for k, c, v in ((3, 0, 0), (11, 1, 0), (20, 1, 1)):
        ev, ec, vv, vc = eigv[k, v], eigv[k, p.nv + c], vec[k, v], vec[k, p.nv + c]
        got = api.optsp_pair(ev, vv, ec, vc, kpt[k], p.cshift, sysm)
        hs = O.hlm(kpt[k], sysm)
        factor = (1.0 / ((ec - ev) + 1j * s32)).real
        for a in range(3):
            want = factor * (np.conj(vc) @ (hs[a] @ vv))
            assert abs(got[a] - want) <= 1e-12 * max(1.0, abs(want)), (k, c, v, a, got[a], want)
    vc3 = O.vcell3D(sysm.rlat)
    E, f = ref["Ws"], ref["acts"]["xx"]
    for rtype in (0, 1):
        for elux in (0.7, 2.31, 4.9):
            rp, ip = api.optdiel(rtype, vc3, p.ngrid, elux, E, f, p.cshift)
            wr, wi = O.optdiel_grid(rtype, vc3, p.ngrid, np.array([elux]), E, f, p.cshift)
            assert abs(rp - wr[0]) <= 1e-12 * max(1.0, abs(wr[0])) and abs(ip - wi[0]) <= 1e-12 * max(1.0, abs(wi[0]))
    for coul, ediel in (("V2DRK", (1.0, 1.0, 1.0)), ("V3DL", (1.0, 8.0, 1.0)), ("V2DK", (1.0, 3.0, 2.0))):
        q = S.BSEParams(**{**p.__dict__})
        q.coultype, q.ediel = coul, ediel
        for i, j in ((0, 7), (3, 3), (12, 30)):
            got = api.coulomb_pair(q, sysm.rlat, kpt[i], kpt[j])
            want = O.coulomb_table(kpt[i:i + 1], kpt[j:j + 1], q, sysm.rlat)[0, 0]
            assert abs(got - want) <= 1e-12 * max(1e-300, abs(want)), (coul, i, j, got, want)


@pytest.mark.parametrize("precision,nev", [("fp64", 100), ("bf16x3", 40), ("fp32", 100)])
def test_more_excitons_than_one_block(ctx, c1, precision, nev):
    """nev beyond one eigensolver block (the reference's bsesolver asks 100, src/module_bse.F90:2432): chunks of 16
    eigenpairs with deflation; every energy within 1e-5 eV of the oracle's dense solve, the spectrum within 1e-4."""
    sysm, p, _ = c1
    q = S.BSEParams(**{**p.__dict__})
    q.nev = nev
    ref = O.bsesolver(sysm, q)
    ctx.set_hr(sysm)
    out = ctx.bsesolver(q, precision=precision, op="matfree")
    err = np.abs(out["E"] - ref["E"])
    assert err.max() <= 1e-5, (precision, nev, err.max(), int(np.argmax(err)))
    assert np.all(np.diff(out["E"]) >= 0)
    spec = O.bsedielraw(out["Ws"], out["acts"], q.ngrid, sysm.rlat, q)
    spec_ref = O.bsedielraw(ref["Ws"], ref["acts"], q.ngrid, sysm.rlat, q)
    for c in ("xx", "yy", "zz"):
        assert rel_l2(spec[c][:, 2], spec_ref[c][:, 2]) <= 1e-4, c


def test_slepc_solver_with_the_reference_ne(ctx, c1):
    """slepc_solver(HX, EX, HE, NX, NE) with the reference's NE = 100: the lowest 100 eigenpairs of the dense matrix,
    eigenvalues within 1e-9 eV of LAPACK's, every residual ||HX x - e x|| / |e| within 1e-8 (SLEPc's tolerance)."""
    sysm, p, ref = c1
    H = O.bse_build(ref["eigv"], ref["vec"], ref["kpt"], p, sysm.rlat)
    EX, HE = ctx.slepc_solver(H, 100)
    w = np.linalg.eigvalsh(H)[:100]
    np.testing.assert_allclose(EX, w, rtol=0, atol=1e-9)
    res = np.linalg.norm(H @ HE - HE * EX[None, :], axis=0) / np.abs(EX)
    assert res.max() <= 1e-8, res.max()
