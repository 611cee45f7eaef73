"""The gradient oracle against central finite differences of the oracle's own forward (CPU only)."""
import copy

import numpy as np
import pytest

from oracle import wtb_oracle_grad as OG
from wtb_gb300 import synthetic as S


def _case(nev=4, seed=3):
    sysm, p = S.workload("hex8_6x6")
    p.nev = nev
    rng = np.random.default_rng(seed)
    return sysm, p, rng.standard_normal(nev), rng.standard_normal(nev), rng


def _fd_hop(sysm, p, a, b, which, r, m, n, h=1e-6):
    sp, sm = copy.deepcopy(sysm), copy.deepcopy(sysm)
    getattr(sp, which)[r, m, n] += h
    getattr(sm, which)[r, m, n] -= h
    return (OG.loss(sp, p, a, b) - OG.loss(sm, p, a, b)) / (2 * h)


def test_grad_oracle_matches_finite_differences():
    sysm, p, a, b, rng = _case()
    dhop, dihop, dr0, _ = OG.backward(sysm, p, a, b)
    for _ in range(6):
        r, m, n = rng.integers(len(sysm.rvec)), rng.integers(sysm.w90basis), rng.integers(sysm.w90basis)
        for which, g in (("hop", dhop), ("ihop", dihop)):
            fd = _fd_hop(sysm, p, a, b, which, r, m, n)
            assert abs(fd - g[r, m, n]) <= 1e-5 * max(abs(fd), 1e-2), (which, r, m, n, fd, g[r, m, n])
    pp, pm = copy.deepcopy(p), copy.deepcopy(p)
    pp.r0 += 1e-4
    pm.r0 -= 1e-4
    fd = (OG.loss(sysm, pp, a, b) - OG.loss(sysm, pm, a, b)) / 2e-4
    assert abs(fd - dr0) <= 1e-5 * max(abs(fd), 1e-2)


def test_grad_oracle_onsite_diagonal_and_upper_triangle():
    """Entries the forward never reads have zero gradient except through H(k): the upper triangle of the
    R = 0 block is read only through its Hermitian partner at -R, and the efermi-shifted diagonal enters
    only through H(k) (not the velocity operator, which drops it)."""
    sysm, p, a, b, rng = _case()
    dhop, dihop, _, _ = OG.backward(sysm, p, a, b)
    r0 = int(np.flatnonzero(np.all(sysm.rvec == 0, axis=1))[0])
    # ihop on the R=0 diagonal only reaches Im of the diagonal, which ZHEEV('L') ignores
    assert np.allclose(np.diag(dihop[r0]), 0.0, atol=1e-12)
    fd = _fd_hop(sysm, p, a, b, "ihop", r0, 1, 1)
    assert abs(fd) < 1e-6


@pytest.mark.parametrize("coul", ["V3DL"])
def test_grad_oracle_r0_zero_for_other_potentials(coul):
    sysm, p, a, b, _ = _case()
    p.coultype = coul
    p.ediel = (1.0, 4.0, 1.0)
    _, _, dr0, _ = OG.backward(sysm, p, a, b)
    assert dr0 == 0.0


def test_grad_oracle_pinned_by_finite_differences_at_dim_5184():
    """The differentiation form at its own size (tests/golden/hex8_36x36_grad_oracle.npz): the gradient oracle's
    gradients of the lowest 4 energies and of the spectrum loss against central differences (h = 1e-6) of the
    oracle's forward on 24 seeded H(R) entries and r0, within 1e-4 relative (floor 1e-3 of the largest entry)."""
    import os

    import numpy as np

    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hex8_36x36_grad_oracle.npz"))
    assert g["fd_entries"].shape == (24, 4) and float(g["fd_h"]) == 1e-6
    for j, k in enumerate(["E0", "E1", "E2", "E3", "spec"]):
        oh, oi = g["dhop_" + k], g["dihop_" + k]
        scale = max(np.abs(oh).max(), np.abs(oi).max())
        for i, (w, r, m, n) in enumerate(g["fd_entries"]):
            v = (oh if w == 0 else oi)[r, m, n]
            assert abs(v - g["fd"][i, j]) <= 1e-4 * max(abs(g["fd"][i, j]), 1e-3 * scale), (k, w, r, m, n)
        assert abs(float(g["dr0_" + k]) - g["fd"][-1, j]) <= 1e-4 * abs(g["fd"][-1, j]), k
