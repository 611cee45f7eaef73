"""Full-size cases, where the CPU oracle is too slow to run per test: the mixed-precision forms against the
plain FP64 GPU form (itself pinned to the oracle on the smaller cases), and the gradient path used to fit a
screening length to a target spectrum made by the oracle (tests/golden/hex8_36x36_fit_target.npz).

Tolerances: exciton energies 1e-5 eV; spectra 1e-4 relative L2; the fitted r0 within 0.3 A of the value the
target was made with (the target carries N(0, 1e-3) noise)."""
import os

import numpy as np
import pytest

from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("name", ["hex12_60x60", "cubic16_16x16x16"])
def test_mixed_precision_against_fp64_at_full_size(ctx, name):
    sysm, p = S.workload(name)
    ctx.set_hr(sysm)
    ref = ctx.bsesolver(p, precision="fp64", op="matfree")
    spec_ref = ctx.bsedielraw(p, ref["Ws"], ref["acts"])
    for prec in ("bf16x3", "fp32"):
        out = ctx.bsesolver(p, precision=prec, op="matfree")
        assert np.max(np.abs(out["E"] - ref["E"])) <= 1e-5, (name, prec, out["E"] - ref["E"])
        # the spectra are sums over these excitons only (rows past nev are zero in both)
        spec = ctx.bsedielraw(p, out["Ws"], out["acts"])
        for c in ("xx", "yy", "zz"):
            assert rel_l2(spec[c][:, 2], spec_ref[c][:, 2]) <= 1e-4, (name, prec, c)
        # E is sorted and the solve reports an FP64 residual of the final block
        assert np.all(np.diff(out["E"]) >= 0)
        assert out["timings"]["max_rel_residual"] < 1e-3


def test_fit_screening_length_to_target_spectrum(ctx):
    """Secant iteration on dL/dr0 = 0 with L the xx least-squares spectrum loss, gradient from
    wtb_spectrum_loss + wtb_bse_backward (bf16x3 forward and backward)."""
    sysm, p = S.workload("hex8_36x36")
    g = np.load(os.path.join(HERE, "golden", "hex8_36x36_fit_target.npz"))
    target, r0_true = g["target"], float(g["r0_true"])
    ctx.set_hr(sysm)
    # the seeded inputs are rebuilt here; LAPACK calls inside the generator may differ in the last bits between
    # machines, so the fixture is checked physically: the FP64 forward at r0_true gives its excitons
    p.r0 = r0_true
    chk = ctx.bsesolver(p, precision="fp64", op="matfree")
    np.testing.assert_allclose(chk["E"], g["E"], atol=1e-6)

    def loss_grad(r0):
        p.r0 = r0
        out = ctx.bsesolver(p, precision="bf16x3", op="matfree")
        L, gE, gf = ctx.spectrum_loss(p, p.dim, out["E"], out["acts"]["xx"][: p.nev], target)
        gr = ctx.bse_backward(p, gE, gf, precision="bf16x3")
        return L, gr["dr0"]

    ra, rb = 40.0, 41.0
    La, ga = loss_grad(ra)
    Lb, gb = loss_grad(rb)
    assert ga < 0  # the loss decreases towards the true r0 = 44
    L0 = La
    for _ in range(8):
        if abs(gb - ga) < 1e-300:
            break
        rc = rb - gb * (rb - ra) / (gb - ga)
        rc = min(max(rc, 30.0), 60.0)
        ra, ga = rb, gb
        rb = rc
        Lb, gb = loss_grad(rb)
        if abs(rb - ra) < 1e-3:
            break
    assert abs(rb - r0_true) < 0.3, rb
    # the target's noise alone leaves numbse * 1e-6 = 1e-3 in the loss
    noise_floor = p.numbse * 1e-6
    assert Lb < L0 and Lb < 1.2 * noise_floor, (Lb, L0)


def test_ipa_spectrum_at_full_size(ctx):
    """spoptics + spdielraw on the 57,600-transition mesh: the records are sorted and hold every (k, c, v)
    once, and the IPA spectrum obeys the Lorentzian sum rule over the window,
    int eps2 = C sum_n f_n [atan((b - E_n)/g) - atan((a - E_n)/g)], g = CSHIFT + avgsme (renormalisation off),
    to the trapezoid rule's 1e-5."""
    from oracle import wtb_oracle as O

    sysm, p = S.workload("hex12_60x60")
    ctx.set_hr(sysm)
    rec = ctx.spoptics(p)
    assert rec.shape == (p.dim, 15)
    assert np.all(np.diff(rec[:, 6]) >= 0)
    nk = p.ngrid[0] * p.ngrid[1] * p.ngrid[2]
    ids = np.unique(np.stack([rec[:, 4] - rec[:, 3], rec[:, 3] - rec[:, 5]], axis=1), axis=0)
    assert len(ids) == p.nc * p.nv
    kid = np.unique(np.round(rec[:, :3].astype(np.float64), 4), axis=0)
    assert len(kid) == nk
    q = S.BSEParams(**{**p.__dict__})
    q.renorm, q.numbse, q.ebse0, q.ebsef = False, 40001, 0.0, 12.0
    esp = rec[:, 6].astype(np.float64)
    acts = {c: rec[:, 7 + i].astype(np.float64) for i, c in enumerate(O.COMPONENTS)}
    d = ctx.spdielraw(q, esp, acts)["xx"]
    spinf = 2.0 if sysm.systype == "NP" else 1.0
    C = O.GAMA / (float(np.float32(nk)) * O.vcell3D(sysm.rlat))
    g = q.cshift + O.avgsme(esp)
    f = acts["xx"]
    expect = spinf * C * np.sum(f * (np.arctan((q.ebsef - esp) / g) - np.arctan((q.ebse0 - esp) / g)))
    integral = np.trapezoid(d[:, 2], d[:, 0])
    assert abs(integral - expect) / expect < 1e-5, (integral, expect)
    assert np.all(np.isfinite(d))
