"""The full-size configurations against the FP64 oracle, per eigenvalue.

The fixtures tests/golden/<workload>_oracle.npz hold the seeded system itself and the oracle's results for
it: the lowest excitons of the FP64 factored operator (the matrix of the reference's element-by-element build,
src/module_bse.F90:2392-2415) from ARPACK at tol 1e-10 in place of SLEPc Krylov-Schur
(src/module_slepc_solver.F90:29-74), two start vectors agreeing to 1e-9 eV, residuals below 1e-8 eV; the
dielbsev/dielbsep activities of those excitons and the three bsedielraw spectra.  Made by
tests/golden/make_golden.py.

Gates (the acceptance bounds): every exciton energy within 1e-5 eV of the oracle's, in every precision form;
the xx, yy, zz spectra within 1e-4 relative L2.  Activities: 1e-4 of the largest in the FP64 forms; in the
reduced-precision forms the eigenvectors carry the 1e-5 residual divided by the smallest gap between the
excitons (9 meV at 57,600), so 2e-2 of the largest.
"""
import os

import numpy as np
import pytest

from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = ["hex12_60x60", "cubic16_16x16x16"]
MODES = [("fp64", "dense"), ("fp64", "matfree"), ("fp32", "matfree"), ("bf16x3", "matfree"), ("bf16x6", "matfree")]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module", params=FIXTURES)
def full(request, ctx):
    name = request.param
    g = np.load(os.path.join(HERE, "golden", name + "_oracle.npz"))
    sysm = S.system_from_arrays(g)
    _, p = S.workload(name, params_only=True)
    ctx.set_hr(sysm)
    return name, sysm, p, g


@pytest.mark.parametrize("precision,op", MODES)
def test_energies_spectra_against_oracle(ctx, full, precision, op):
    name, sysm, p, g = full
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision=precision, op=op)
    dE = np.abs(out["E"] - g["E"])
    spec = ctx.bsedielraw(p, out["Ws"], out["acts"])
    sl2 = {c: rel_l2(spec[c][:, 2], g["spec_" + c][:, 2]) for c in ("xx", "yy", "zz")}
    t = out["timings"]
    print(f"{name} {precision}/{op}: |dE| vs oracle (eV) = {np.array2string(dE, precision=2)}; spectrum rel L2 "
          f"{ {c: f'{v:.2e}' for c, v in sl2.items()} }; iterations {t['iterations']}, residual "
          f"{t['max_rel_residual']:.2e}")
    assert dE.shape == (p.nev,)
    assert np.all(dE <= 1e-5), (name, precision, op, dE)
    for c in ("xx", "yy", "zz"):
        np.testing.assert_array_equal(spec[c][:, 0], g["spec_" + c][:, 0])
        assert rel_l2(spec[c][:, 2], g["spec_" + c][:, 2]) <= 1e-4, (name, precision, op, c)
        assert rel_l2(spec[c][:, 1], g["spec_" + c][:, 1]) <= 1e-4, (name, precision, op, c)
    tol = 1e-4 if precision == "fp64" else 2e-2
    for c in ("xx", "yy", "zz", "xy", "sp", "sm"):
        ref = g["act_" + c]
        scale = max(np.abs(ref).max(), 1e-300)
        assert np.max(np.abs(out["acts"][c][: p.nev] - ref)) <= tol * scale, (name, precision, op, c)


def test_fft_operator_at_full_size(ctx):
    """The FP32 matrix-free operator of the 60 x 60 mesh is the FFT convolution (P = 128): 16 applications against
    the oracle's FP64 factored operator, relative to ||H x||."""
    from oracle import wtb_oracle as O

    g = np.load(os.path.join(HERE, "golden", "hex12_60x60_oracle.npz"))
    sysm = S.system_from_arrays(g)
    _, p = S.workload("hex12_60x60", params_only=True)
    ctx.set_hr(sysm)
    ctx.bsesolver(p, precision="fp32", op="matfree")  # stages the mesh and its bands
    kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
    eigv, vec, _ = O.bands(sysm, p, kpt)
    rng = np.random.default_rng(128)
    X = rng.normal(size=(p.dim, 16)) + 1j * rng.normal(size=(p.dim, 16))
    Y = ctx.bse_matvec(p, X, precision="fp32", op="matfree")
    assert ctx.operator_form() == "FP32 FFT convolution"
    Yref = O.bse_matvec_factored(X, eigv, O.gauge_fix(vec), kpt, p, sysm.rlat)
    err = np.linalg.norm(Y - Yref, axis=0) / np.linalg.norm(Yref, axis=0)
    print(f"hex12_60x60 FFT operator: max relative error {err.max():.2e}")
    assert err.max() <= 2e-6, err
