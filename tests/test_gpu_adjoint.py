"""wtb_bse_backward / wtb_spectrum_loss (through the C ABI) against the gradient oracle, which is itself
pinned to finite differences of the forward oracle (tests/test_oracle_grad.py), and against finite
differences of the library's own FP64 forward.

Tolerances: FP64 gradients 1e-6 of the largest |dL/dhop| entry (the adjoint solve stops at 1e-10 relative
residual, the forward eigensolve at 1e-8); mixed-precision gradients 1e-4 relative in the Frobenius norm;
spectrum loss 1e-10 relative, its cotangents 1e-5 relative to central differences."""
import copy

import numpy as np
import pytest

from oracle import wtb_oracle as O
from oracle import wtb_oracle_grad as OG
from wtb_gb300 import api
from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def small_grad():
    sysm, p = S.workload("hex8_6x6")
    p.nev = 4
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal(p.nev), rng.standard_normal(p.nev)
    dhop, dihop, dr0, d = OG.backward(sysm, p, a, b)
    return sysm, p, a, b, dhop, dihop, dr0, d


@pytest.mark.parametrize("op", ["dense", "matfree"])
def test_backward_fp64_matches_gradient_oracle(ctx, small_grad, op):
    sysm, p, a, b, dhop, dihop, dr0, d = small_grad
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision="fp64", op=op)
    np.testing.assert_allclose(out["E"], d["E"], atol=1e-9)
    g = ctx.bse_backward(p, a, b, precision="fp64")
    scale = max(np.max(np.abs(dhop)), np.max(np.abs(dihop)))
    assert np.max(np.abs(g["dhop"] - dhop)) <= 1e-6 * scale
    assert np.max(np.abs(g["dihop"] - dihop)) <= 1e-6 * scale
    assert abs(g["dr0"] - dr0) <= 1e-6 * max(abs(dr0), 1e-3)
    assert g["timings"]["iterations"] > 0


def test_backward_energy_only_needs_no_adjoint_solve(ctx, small_grad):
    sysm, p, a, _, _, _, _, d = small_grad
    dhop, dihop, dr0, _ = OG.backward(sysm, p, a, np.zeros(p.nev), d=d)
    ctx.set_hr(sysm)
    ctx.bsesolver(p, precision="fp64", op="matfree")
    g = ctx.bse_backward(p, a, None, precision="fp64")
    assert g["timings"]["iterations"] == 0
    scale = max(np.max(np.abs(dhop)), np.max(np.abs(dihop)))
    assert np.max(np.abs(g["dhop"] - dhop)) <= 1e-6 * scale
    assert np.max(np.abs(g["dihop"] - dihop)) <= 1e-6 * scale
    assert abs(g["dr0"] - dr0) <= 1e-6 * max(abs(dr0), 1e-3)


def test_backward_matches_finite_differences_of_the_gpu_forward(ctx, small_grad):
    sysm, p, a, b, _, _, _, _ = small_grad
    ctx.set_hr(sysm)
    ctx.bsesolver(p, precision="fp64", op="dense", tol=1e-12)
    g = ctx.bse_backward(p, a, b, precision="fp64")

    def L(s, q):
        ctx.set_hr(s)
        o = ctx.bsesolver(q, precision="fp64", op="dense", tol=1e-12)
        return float(a @ o["E"] + b @ o["acts"]["xx"][: q.nev])

    rng = np.random.default_rng(5)
    h = 1e-5
    for _ in range(3):
        r, m, n = rng.integers(len(sysm.rvec)), rng.integers(sysm.w90basis), rng.integers(sysm.w90basis)
        for which, key in (("hop", "dhop"), ("ihop", "dihop")):
            sp, sm = copy.deepcopy(sysm), copy.deepcopy(sysm)
            getattr(sp, which)[r, m, n] += h
            getattr(sm, which)[r, m, n] -= h
            fd = (L(sp, p) - L(sm, p)) / (2 * h)
            assert abs(fd - g[key][r, m, n]) <= 1e-4 * max(abs(fd), 1e-1), (which, r, m, n, fd, g[key][r, m, n])
    pp, pm = copy.deepcopy(p), copy.deepcopy(p)
    pp.r0 += 1e-4
    pm.r0 -= 1e-4
    fd = (L(sysm, pp) - L(sysm, pm)) / 2e-4
    assert abs(fd - g["dr0"]) <= 1e-4 * max(abs(fd), 1e-3)
    ctx.set_hr(sysm)


@pytest.fixture(scope="module")
def c1_grad(ctx):
    sysm, p = S.workload("hex8_24x24")
    rng = np.random.default_rng(7)
    a, b = rng.standard_normal(p.nev), rng.standard_normal(p.nev)
    ctx.set_hr(sysm)
    ctx.bsesolver(p, precision="fp64", op="matfree")
    g64 = ctx.bse_backward(p, a, b, precision="fp64")
    return sysm, p, a, b, g64


@pytest.mark.parametrize("prec", ["fp32", "bf16x3", "bf16x6"])
def test_backward_mixed_precision_against_fp64(ctx, c1_grad, prec):
    sysm, p, a, b, g64 = c1_grad
    ctx.set_hr(sysm)
    ctx.bsesolver(p, precision=prec, op="matfree")
    g = ctx.bse_backward(p, a, b, precision=prec)
    for key in ("dhop", "dihop"):
        err = np.linalg.norm(g[key] - g64[key]) / np.linalg.norm(g64[key])
        print(f"{prec} {key}: relative Frobenius error against FP64 {err:.2e}")
        assert err <= 1e-4, (prec, key, err)
    print(f"{prec} dr0: relative error against FP64 {abs(g['dr0'] - g64['dr0']) / abs(g64['dr0']):.2e}")
    assert abs(g["dr0"] - g64["dr0"]) <= 1e-4 * abs(g64["dr0"])


def test_spectrum_loss_and_chain_rule(ctx, small_grad):
    sysm, p, _, _, _, _, _, d = small_grad
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision="fp64", op="dense")
    E, f = out["E"], out["acts"]["xx"][: p.nev]
    dimse = p.dim
    vc = O.vcell3D(sysm.rlat)
    spinf = 2.0 if sysm.systype == "NP" else 1.0
    rng = np.random.default_rng(11)
    omega = np.linspace(p.ebse0, p.ebsef, p.numbse)
    target = 0.5 * np.exp(-((omega - 2.5) / 0.4) ** 2) + 0.01 * rng.standard_normal(p.numbse)
    L, gE, gf = ctx.spectrum_loss(p, dimse, E, f, target)
    L_ref = OG.spectrum_loss(E, f, dimse, p, vc, target, spinf)
    assert abs(L - L_ref) <= 1e-10 * abs(L_ref)
    for n in range(p.nev):
        for arr, g in ((E, gE), (f, gf)):
            h = 1e-7 * max(1.0, abs(arr[n]))
            ap, am = arr.copy(), arr.copy()
            ap[n] += h
            am[n] -= h
            Ep, fp = (ap, f) if arr is E else (E, ap)
            Em, fm = (am, f) if arr is E else (E, am)
            fd = (OG.spectrum_loss(Ep, fp, dimse, p, vc, target, spinf) -
                  OG.spectrum_loss(Em, fm, dimse, p, vc, target, spinf)) / (2 * h)
            assert abs(fd - g[n]) <= 1e-5 * max(abs(fd), 1e-3 * max(1.0, abs(L_ref))), (n, fd, g[n])
    # the chain: d(spectrum loss)/dH(R) through wtb_bse_backward equals the oracle's with the same cotangents
    g = ctx.bse_backward(p, gE, gf, precision="fp64")
    dhop, dihop, _, _ = OG.backward(sysm, p, gE, gf, d=d)
    scale = max(np.max(np.abs(dhop)), np.max(np.abs(dihop)))
    assert np.max(np.abs(g["dhop"] - dhop)) <= 1e-6 * scale
    assert np.max(np.abs(g["dihop"] - dihop)) <= 1e-6 * scale


def test_backward_state_and_argument_errors(ctx, small_grad):
    sysm, p, a, b, _, _, _, _ = small_grad
    ctx.set_hr(sysm)
    with pytest.raises(api.WTBError) as e:
        ctx.bse_backward(p, a, b)
    assert e.value.code == api.STATUS["WTB_ESTATE"]
    ctx.bsesolver(p, precision="fp64", op="dense")
    q = copy.deepcopy(p)
    q.r0 = p.r0 * 1.5
    with pytest.raises(api.WTBError) as e:
        ctx.bse_backward(q, a, b)
    assert e.value.code == api.STATUS["WTB_EBADARG"]
    with pytest.raises(api.WTBError) as e:
        ctx.bse_backward(p, a, b, precision="fp32")
    assert e.value.code == api.STATUS["WTB_EBADARG"]
    bad = a.copy()
    bad[0] = np.nan
    with pytest.raises(api.WTBError) as e:
        ctx.bse_backward(p, bad, b)
    assert e.value.code == api.STATUS["WTB_ENAN"]
