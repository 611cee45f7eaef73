"""wtb_batch_* against single-context solves and the oracle.

The split-BF16 forms run as one joint eigensolve over all systems (one graph launch); the other forms system
by system.  Tolerances: FP64 batch vs single-context solve 1e-9 eV (the same kernels, only reduction orders
may differ); bf16x3 batch vs single-context solve 2e-6 eV and activities 1e-4 relative to the largest (the
joint solve sums its reductions over other row ranges, so each system follows its own rounding path to the
same split-BF16 accuracy, about 1e-7 eV from FP64); against the oracle 1e-5 eV, activities 1e-4 relative to
the largest."""
import numpy as np
import pytest

from oracle import wtb_oracle as O
from wtb_gb300 import api
from wtb_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def items():
    full = S.strained_batch(nsys=64)
    # the 6 smallest systems of the C4 batch keep the test short
    order = sorted(range(len(full)), key=lambda i: full[i][1].dim)
    return [full[i] for i in order[:6]]


@pytest.mark.parametrize("prec", ["fp64", "bf16x3"])
def test_batch_matches_single_context(ctx, items, prec):
    b = api.Batch(0, nworkers=4)
    try:
        out, wall = b.bsesolver(items, precision=prec, op="matfree")
    finally:
        b.close()
    assert wall > 0
    for (s, p), o in zip(items, out):
        assert o["status"] == 0 and o["iterations"] > 0
        ctx.set_hr(s)
        ref = ctx.bsesolver(p, precision=prec, op="matfree")
        tol_e, tol_a = (1e-9, 1e-9) if prec == "fp64" else (2e-6, 1e-4)
        np.testing.assert_allclose(o["E"], ref["E"], atol=tol_e)
        for c in ("xx", "yy", "sp"):
            np.testing.assert_allclose(o["acts"][c], ref["acts"][c][: p.nev], atol=tol_a * max(1.0, np.abs(ref["acts"][c]).max()))


def test_joint_batch_relaunch_and_uneven_sizes(ctx):
    """The cached batch graph relaunched gives the same results; a batch mixing the smallest and largest C4
    systems (576 and 11,664 rows) matches the single-context solves."""
    full = S.strained_batch(nsys=64)
    order = sorted(range(len(full)), key=lambda i: full[i][1].dim)
    items = [full[i] for i in (order[0], order[1], order[-1], order[len(order) // 2])]
    b = api.Batch(0, nworkers=1)
    try:
        out1, _ = b.bsesolver(items, precision="bf16x3", op="matfree")
        out2, _ = b.bsesolver(items, precision="bf16x3", op="matfree")
    finally:
        b.close()
    for (s, p), o1, o2 in zip(items, out1, out2):
        np.testing.assert_array_equal(o1["E"], o2["E"])
        ctx.set_hr(s)
        ref = ctx.bsesolver(p, precision="bf16x3", op="matfree")
        np.testing.assert_allclose(o1["E"], ref["E"], atol=2e-6)


def test_batch_against_oracle(items):
    b = api.Batch(0, nworkers=3)
    try:
        out, _ = b.bsesolver(items[:3], precision="bf16x3", op="matfree")
    finally:
        b.close()
    for (s, p), o in zip(items[:3], out):
        ref = O.bsesolver(s, p)
        np.testing.assert_allclose(o["E"], ref["E"], atol=1e-5)
        fx = ref["acts"]["xx"][: p.nev]
        np.testing.assert_allclose(o["acts"]["xx"], fx, atol=1e-4 * np.abs(fx).max())


def test_batch_reports_failing_system_and_finishes_the_rest(items):
    bad_s, bad_p = items[0][0].copy(), items[0][1]
    bad_s.efermi = -1e3  # no occupied band: "Number of valence states higher then ocuppied states"
    batch = [items[1], (bad_s, bad_p), items[2]]
    b = api.Batch(0, nworkers=2)
    try:
        out, _ = b.bsesolver(batch, precision="bf16x3", op="matfree", raise_on_error=False)
        with pytest.raises(api.WTBError):
            b.bsesolver(batch, precision="bf16x3", op="matfree")
    finally:
        b.close()
    assert out[0]["status"] == 0 and out[2]["status"] == 0
    assert out[1]["status"] != 0
    assert "valence" in out[1]["error"]


def test_joint_batch_host_driven_loop_matches_graph(items):
    """WTB_SOLVER_STREAM runs the joint solve without a graph (kernel profilers cannot see inside conditional
    graph bodies): the same kernels in the same order, so the same results."""
    import os
    b = api.Batch(0)
    try:
        g, _ = b.bsesolver(items[:4])
        os.environ["WTB_SOLVER_STREAM"] = "1"
        try:
            e, _ = b.bsesolver(items[:4])
        finally:
            del os.environ["WTB_SOLVER_STREAM"]
        g2, _ = b.bsesolver(items[:4])  # back to a (rebuilt) graph
    finally:
        b.close()
    for a, c, d in zip(g, e, g2):
        np.testing.assert_allclose(c["E"], a["E"], atol=1e-12)
        np.testing.assert_allclose(d["E"], a["E"], atol=1e-12)


def test_batch_matvec_matches_single_context(ctx, items):
    """The joint operator (one gather, one grouped contraction, one scatter launch over all systems) applied
    to random blocks equals each system's own operator to FP32 rounding."""
    rng = np.random.default_rng(5)
    sub = items[:3]
    b = api.Batch(0)
    try:
        b.bsesolver(sub)
        Xs = [rng.standard_normal((p.dim, 4)) + 1j * rng.standard_normal((p.dim, 4)) for _, p in sub]
        Ys = b.matvec(Xs)
    finally:
        b.close()
    for (s, p), X, Y in zip(sub, Xs, Ys):
        ctx.set_hr(s)
        ctx.bsesolver(p, precision="bf16x3", op="matfree")
        Yr = ctx.bse_matvec(p, X, precision="bf16x3", op="matfree")
        assert np.abs(Y - Yr).max() <= 1e-6 * np.abs(Yr).max()
