"""The differentiation form at its own size: hex8_36x36 (2D hexagonal w=8, 36x36x1, 2v+2c, BSE dim 5184, lowest 4
excitons, V2DRK r0 = 40 A).  Gradients of five losses -- each of the lowest 4 exciton energies and the L2 spectrum
loss against the fitting case's seeded target spectrum -- with respect to every H(R) entry (hopmatrices and
ihopmatrices) and r0, through wtb_bse_backward (and wtb_spectrum_loss for the spectrum loss's cotangents), in
FP64 and in the mixed-precision forms.

References, both from tests/golden/hex8_36x36_grad_oracle.npz (tests/golden/make_golden.py):
  * the FP64 gradient oracle (oracle/wtb_oracle_grad.py) on every entry and r0;
  * central finite differences (step 1e-6) of the oracle's FP64 forward on 24 seeded H(R) entries and on r0.

Tolerances: FP64 -- every entry within 1e-6 of the largest gradient entry of the oracle, and within 1e-4 of the
finite difference (relative, with a floor of 1e-3 of the largest entry for entries whose gradient is small).
Mixed precision -- the relative Frobenius error against the oracle's gradient over all entries, the relative
L2 error against the finite differences over the sampled entries, and r0's relative error, each within 1e-4.
"""
import os

import numpy as np
import pytest

from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
LOSSES = ["E0", "E1", "E2", "E3", "spec"]


@pytest.fixture(scope="module")
def c5():
    g = np.load(os.path.join(HERE, "golden", "hex8_36x36_grad_oracle.npz"))
    sysm = S.system_from_arrays(g)
    _, p = S.workload("hex8_36x36", params_only=True)
    return sysm, p, g


def gradients(ctx, sysm, p, g, precision, tol):
    """The five gradients (dhop, dihop, dr0) through the library, with the forward solved once."""
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision=precision, op="matfree", tol=tol)
    res = {"E": out["E"], "residual": out["timings"]["max_rel_residual"]}
    for key in LOSSES:
        if key == "spec":
            L, gE, gf = ctx.spectrum_loss(p, p.dim, out["E"], out["acts"]["xx"][: p.nev], g["target"])
            res["spec_loss"] = L
            gr = ctx.bse_backward(p, gE, gf, precision=precision)
        else:
            gr = ctx.bse_backward(p, np.eye(p.nev)[int(key[1])], None, precision=precision)
        res[key] = gr
    return res


def errors(res, g):
    """Per loss: the largest entry error against the oracle's gradient over the largest oracle entry, the
    Frobenius error over the oracle's norm, the r0 error, and the worst relative error against the finite
    differences (floor 1e-3 of the largest entry)."""
    out = {}
    ent = g["fd_entries"]
    for j, key in enumerate(LOSSES):
        gr = res[key]
        oh, oi, orr = g[f"dhop_{key}"], g[f"dihop_{key}"], float(g[f"dr0_{key}"])
        scale = max(np.abs(oh).max(), np.abs(oi).max())
        emax = max(np.abs(gr["dhop"] - oh).max(), np.abs(gr["dihop"] - oi).max()) / scale
        frob = np.sqrt(np.sum((gr["dhop"] - oh) ** 2) + np.sum((gr["dihop"] - oi) ** 2)) / \
            np.sqrt(np.sum(oh ** 2) + np.sum(oi ** 2))
        fd_rel = 0.0
        got_s, fd_s = [], []
        for i, (which, r, m, n) in enumerate(ent):
            v = (gr["dhop"] if which == 0 else gr["dihop"])[r, m, n]
            fd = g["fd"][i, j]
            fd_rel = max(fd_rel, abs(v - fd) / max(abs(fd), 1e-3 * scale))
            got_s.append(v)
            fd_s.append(fd)
        got_s, fd_s = np.array(got_s), np.array(fd_s)
        fd = g["fd"][len(ent), j]
        r0_fd = abs(gr["dr0"] - fd) / max(abs(fd), 1e-12)
        out[key] = {"max_vs_oracle": emax, "frob_vs_oracle": frob, "r0_vs_oracle": abs(gr["dr0"] - orr) / max(abs(orr), 1e-12),
                    "max_vs_fd": fd_rel, "l2_vs_fd": float(np.linalg.norm(got_s - fd_s) / np.linalg.norm(fd_s)),
                    "r0_vs_fd": r0_fd}
    return out


def report(tag, res, err):
    print(f"\n{tag}: forward residual {res['residual']:.2e}")
    for key, e in err.items():
        print(f"  {key:5s} vs oracle max {e['max_vs_oracle']:.2e} frob {e['frob_vs_oracle']:.2e} r0 {e['r0_vs_oracle']:.2e}"
              f" | vs FD max {e['max_vs_fd']:.2e} l2 {e['l2_vs_fd']:.2e} r0 {e['r0_vs_fd']:.2e}")


def test_fixture_energies(ctx, c5):
    """The GPU's FP64 forward on the stored system gives the oracle's lowest 4 excitons."""
    sysm, p, g = c5
    ctx.set_hr(sysm)
    out = ctx.bsesolver(p, precision="fp64", op="matfree", tol=1e-12)
    np.testing.assert_allclose(out["E"], g["E"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(out["acts"]["xx"][: p.nev], g["f"], rtol=1e-7, atol=0)


def test_fp64_gradients_against_oracle_and_finite_differences(ctx, c5):
    sysm, p, g = c5
    res = gradients(ctx, sysm, p, g, "fp64", 1e-12)
    err = errors(res, g)
    report("fp64", res, err)
    for key, e in err.items():
        assert e["l2_vs_fd"] <= 1e-5, (key, e)
        assert e["max_vs_oracle"] <= 1e-6, (key, e)
        assert e["r0_vs_oracle"] <= 1e-6, (key, e)
        assert e["max_vs_fd"] <= 1e-4, (key, e)
        assert e["r0_vs_fd"] <= 1e-4, (key, e)


@pytest.mark.parametrize("precision", ["bf16x3", "bf16x6"])
def test_mixed_precision_gradients(ctx, c5, precision):
    """Mixed precision at the library's default forward target (1e-5) and at 1e-7: every loss's gradient within
    1e-4 relative of the oracle's (Frobenius over all entries), of the finite differences (L2 over the sampled
    entries) and of r0's finite difference.  Measured on a GB300: 3e-7 (energies) and 3e-5 (spectrum loss) from
    the oracle; the entrywise error is printed as well -- it is 4e-7 of the largest entry, so entries near zero
    carry larger relative errors than the norms."""
    sysm, p, g = c5
    for tol in (0.0, 1e-7):
        res = gradients(ctx, sysm, p, g, precision, tol)
        err = errors(res, g)
        report(f"{precision} tol {tol or 'default'}", res, err)
        for key, e in err.items():
            assert e["frob_vs_oracle"] <= 1e-4, (precision, tol, key, e)
            assert e["l2_vs_fd"] <= 1e-4, (precision, tol, key, e)
            assert e["r0_vs_fd"] <= 1e-4, (precision, tol, key, e)
