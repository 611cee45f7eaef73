"""The output writers (host code of the library, no GPU): every formatted record against the oracle's
restatement of the Fortran edit descriptors, whole files byte for byte, and the read-back that PP_ONLY runs do."""
import os

import numpy as np
import pytest

from oracle import wtb_oracle as O

COMPS = ("xx", "yy", "zz", "xy", "xz", "yz", "sp", "sm")


def _values(rng, n):
    mag = 10.0 ** rng.uniform(-9, 12, n)
    v = np.where(rng.random(n) < 0.5, -mag, mag)
    edge = [0.0, -0.0, 0.5, 1.03125, -1.03125, 0.00005, 0.00015, 9.99995, 99999999.99995, 1e10, 9.99996e-5,
            1.0e-99, 1.0e-100, 1.0e100, 123.456789, float(np.float32(1.9297071)), np.inf, -np.inf, np.nan]
    return np.concatenate([v, edge])


@pytest.mark.parametrize("kind,w,d", [("F", 15, 4), ("F", 10, 4), ("E", 15, 4), ("F", 6, 4), ("E", 10, 4)])
def test_edit_descriptors_match_restatement(built, kind, w, d):
    from wtb_gb300 import api

    rng = np.random.default_rng(7)
    ref = O.fortran_F if kind == "F" else O.fortran_E
    for x in _values(rng, 3000):
        assert api.fortran_format(kind, x, w, d) == ref(x, w, d), (kind, w, d, repr(x))


def test_integer_descriptor(built):
    from wtb_gb300 import api

    for v, w, m in [(0, 10, 0), (0, 12, 1), (7, 10, 0), (-17, 12, 1), (123456789012, 10, 0), (42, 3, 1)]:
        assert api.fortran_format("I", v, w, m) == O.fortran_I(v, w, m)


def _read_table(path, skip):
    with open(path) as f:
        lines = f.read().splitlines()[skip:]
    return np.array([[float(t) for t in ln.split()] for ln in lines])


def test_bse_opt_diel_files(built, tmp_path):
    from wtb_gb300 import api

    rng = np.random.default_rng(3)
    dim = 57
    Ws = np.sort(rng.uniform(1.0, 4.0, dim))
    Ws[10:] = 0.0                                      # rows past nev, as bsesolver leaves them
    acts = {c: np.where(np.arange(dim) < 10, rng.uniform(-2, 50, dim), 0.0) for c in COMPS}
    for pol in (False, True):
        path = os.path.join(tmp_path, "bse_opt_diel-pol.dat" if pol else "bse_opt_diel.dat")
        api.write_bse_opt_diel(path, Ws, acts, pol)
        cols = ("xx", "yy", "zz", "sp", "sm") if pol else COMPS[:6]
        head = (" #  exciton energy  xx  yy  zz sp  sm" if pol else " #  exciton energy  xx  yy  zz xy  xz  yz")
        expect = [head] + ["".join([O.fortran_F(Ws[i], 15, 4)] + [O.fortran_F(acts[c][i], 15, 4) for c in cols])
                           for i in range(dim)]
        assert open(path).read() == "\n".join(expect) + "\n"
        back = _read_table(path, 1)                    # what bsedielraw's list-directed read recovers
        np.testing.assert_allclose(back[:, 0], Ws, atol=5e-5)
        np.testing.assert_allclose(back[:, 1], acts["xx"], atol=5e-5)


def test_sp_optics_and_tm_coef_files(built, tmp_path):
    from wtb_gb300 import api

    rng = np.random.default_rng(4)
    nk, nc, nv = 9, 2, 3
    dim = nk * nc * nv
    rec = rng.uniform(-1, 3, (dim, 15)).astype(np.float32)
    rec[:, 3:6] = rng.integers(0, 12, (dim, 3))
    rec[0, 3:6] = 0                                    # I10.0 of zero is a blank field
    api.write_sp_optics(os.path.join(tmp_path, "sp.dat"), rec)
    api.write_tm_coef(os.path.join(tmp_path, "tm.dat"), nk, nc, nv, rec)
    api.write_tm_coef(os.path.join(tmp_path, "tmp.dat"), nk, nc, nv, rec, pol=True)
    sp = [" #  energy  xx  yy  zz  xy  xz  yz"] + ["".join(O.fortran_F(float(rec[i, c]), 15, 4) for c in range(6, 13))
                                                 for i in range(dim)]
    assert open(os.path.join(tmp_path, "sp.dat")).read() == "\n".join(sp) + "\n"
    for name, cols in (("tm.dat", list(range(6, 13))), ("tmp.dat", [6, 7, 8, 9, 13, 14])):
        lines = open(os.path.join(tmp_path, name)).read().splitlines()
        assert lines[0] == " number of kpoints:" + O.fortran_I(nk, 12)
        assert lines[1] == " number of conduction states" + O.fortran_I(nc, 12)
        for i in range(dim):
            want = ("".join(O.fortran_F(float(rec[i, c]), 10, 4) for c in range(3))
                    + "".join(O.fortran_I(int(rec[i, c]), 10, 0) for c in range(3, 6))
                    + "".join(O.fortran_F(float(rec[i, c]), 10, 4) for c in cols))
            assert lines[4 + i] == want
    assert lines[4][30:60] == " " * 30                 # the zero integers of row 0


def test_exc_wf_and_lifetime_files(built, tmp_path):
    from wtb_gb300 import api

    rng = np.random.default_rng(5)
    nk, nc, nv = 4, 2, 2
    nocp = np.full(nk, 6, dtype=np.int32)
    kpt = rng.uniform(-1, 1, (nk, 3))
    ewf = (rng.standard_normal(nk * nc * nv) + 1j * rng.standard_normal(nk * nc * nv)) * 1e-3
    path = os.path.join(tmp_path, "exc_wf_3.dat")
    api.write_exc_wf(path, nocp, kpt, nc, nv, 3, 2.5, ewf)
    lines = open(path).read().splitlines()
    assert lines[0] == " # excitonic state" + O.fortran_I(3, 12)
    assert lines[1] == O.list_directed_record([("c", "#"), ("c", " "), ("c", "exciton energy:"), ("r8", 2.5)])
    assert lines[2] == O.list_directed_record([("c", "#"), ("c", " "), ("c", "number occupied states"), ("i", 6),
                                               ("c", "(not valid for metallic systems)")])
    I = 0
    for k in range(nk):
        for c in range(nc):
            for v in range(nv):
                want = (O.fortran_I(nocp[k], 12) + "".join(O.fortran_F(kpt[k, d], 15, 4) for d in range(3))
                        + O.fortran_I(nocp[k] + c + 1, 12) + O.fortran_I(nocp[k] - nv + v + 1, 12)
                        + O.fortran_E(ewf[I].real, 15, 4) + O.fortran_E(ewf[I].imag, 15, 4))
                assert lines[7 + I] == want
                I += 1
    e = np.array([1.5, 2.0, 0.0])
    lft = np.array([[1e-12, 2e-12, 3e-12, np.inf], [4e-9, 5e-9, 6e-9, 7e-9], [np.inf] * 4]).T.copy()
    lft = lft.T
    path = os.path.join(tmp_path, "exciton_lifetime.dat")
    api.write_exciton_lifetime(path, e, lft)
    lines = open(path).read().splitlines()
    assert lines[0] == " #energy(eV) sum-lft(s)  x-lft(s) y-lft(s) z-lft(s)"
    for i in range(3):
        assert lines[1 + i] == O.fortran_F(e[i], 15, 4) + "".join(O.fortran_E(lft[i, c], 15, 4) for c in range(4))
    assert "Infinity" in lines[3]


def test_writer_rejects_unwritable_path(built):
    from wtb_gb300 import api

    with pytest.raises(api.WTBError):
        api.write_exciton_lifetime("/nonexistent-dir/x.dat", np.ones(2), np.ones((2, 4)))


def test_lifetime_pol_file(built, tmp_path):
    from wtb_gb300 import api

    e = np.array([1.5, 2.25])
    lft = np.array([[1e-12, 2e-12, 3e-12, 4e-12, 5e-12, 6e-12], [7e-9, 8e-9, 9e-9, np.inf, 1e-8, 2e-8]])
    path = os.path.join(tmp_path, "exciton_lifetime-pol.dat")
    api.write_exciton_lifetime(path, e, lft, pol=True)
    lines = open(path).read().splitlines()
    assert lines[0] == " #energy(eV) sum-lft(s)  x-lft(s) y-lft(s) z-lft(s) sp-lft(s) sm-lft(s)"
    for i in range(2):
        assert lines[1 + i] == O.fortran_F(e[i], 15, 4) + "".join(O.fortran_E(lft[i, c], 15, 4) for c in range(6))


def test_exc_wf_finite_q_header(built, tmp_path):
    from wtb_gb300 import api

    path = os.path.join(tmp_path, "exc_wf_2_5.dat")
    api.write_exc_wf(path, np.full(2, 4, dtype=np.int32), np.zeros((2, 3)), 1, 1, 2, 1.75, np.ones(2, complex),
                     q4=[0.25, 0.1, -0.2, 0.0])
    lines = open(path).read().splitlines()
    assert lines[0] == O.list_directed_record([("c", "#"), ("c", " "), ("c", "excitonic momentum"), ("r4", 0.1),
                                               ("r4", -0.2), ("r4", 0.0)])
    assert [float(t) for t in lines[0].split()[3:]] == [np.float32(0.1), np.float32(-0.2), 0.0]
    assert lines[1] == " # excitonic state" + O.fortran_I(2, 12)
    assert len(lines) == 8 + 2


def _ld_values(rng, n, kind):
    mag = 10.0 ** rng.uniform(-40 if kind == 4 else -300, 38 if kind == 4 else 300, n)
    v = np.where(rng.random(n) < 0.5, -mag, mag)
    d = 17 if kind == 8 else 9
    b = [0.1, 10.0 ** d, 1.0, 10.0, 0.5]                # the G rule's F / E boundaries and neighbours
    if kind == 8:
        edge = [x for c in b for x in (np.nextafter(c, 0), c, np.nextafter(c, np.inf))]
    else:
        edge = [float(x) for c in b for x in (np.nextafter(np.float32(c), np.float32(0)), np.float32(c),
                                                np.nextafter(np.float32(c), np.float32(np.inf)))]
    edge += [0.0, -0.0, 1.03125, 123.456, 1e-3, 5e-324, 1.7976931348623157e308, np.inf, -np.inf, np.nan]
    if kind == 4:
        edge = [x for x in edge if not np.isfinite(x) or abs(x) < 3.4e38]
    return np.concatenate([v, np.array(edge)])


@pytest.mark.parametrize("kind", [8, 4])
def test_list_directed_items_match_restatement(built, kind):
    from wtb_gb300 import api

    rng = np.random.default_rng(11 + kind)
    w, d = (25, 17) if kind == 8 else (16, 9)
    for x in _ld_values(rng, 3000, kind):
        assert api.fortran_format("G", x, w, d) == O.list_directed_real(x, kind), (kind, repr(x))


def test_list_directed_known_outputs(built):
    """gfortran's list-directed output of a few values (a blank, then the item's field)."""
    from wtb_gb300 import api

    known8 = {1.0: "   1.0000000000000000     ", 0.1: "  0.10000000000000001     ",
              1e-3: "   1.0000000000000000E-003", -1.0: "  -1.0000000000000000     ",
              0.0: "   0.0000000000000000     ", 123.456: "   123.45600000000000     "}
    known4 = {1.0: "   1.00000000    ", 0.1: "  0.100000001    ", 1e-3: "   1.00000005E-03"}
    for x, s in known8.items():
        assert O.list_directed_record([("r8", x)]) == s
        assert " " + api.fortran_format("G", x, 25, 17) == s
    for x, s in known4.items():
        assert O.list_directed_record([("r4", x)]) == s
        assert " " + api.fortran_format("G", x, 16, 9) == s
    assert O.list_directed_record([("i", 1), ("i", -2)]) == "           1          -2"
    assert O.list_directed_record([("c", "#"), ("c", "  "), ("c", "energy"), ("i", 3), ("c", "x")]) == \
        " #  energy           3 x"
    assert O.list_directed_record([]) == ""
    with pytest.raises(api.WTBError):                     # only the two list-directed real kinds exist
        api.fortran_format("G", 1.0, 20, 10)


def test_list_directed_files(built, tmp_path):
    from wtb_gb300 import api

    rng = np.random.default_rng(12)
    numbse = 41
    dielf = np.stack([np.linspace(0.0, 6.0, numbse), rng.uniform(-3, 30, numbse), rng.uniform(0, 25, numbse)], 1)
    dielf[3, 2] = 1e-7                                    # an E-form item
    path = os.path.join(tmp_path, "bse_diel_xx.dat")
    api.write_diel(path, dielf)
    want = [O.list_directed_record([("c", "#"), ("c", "  "), ("c", "energy"), ("c", "  "), ("c", "real"),
                                    ("c", "  "), ("c", "imag")])]
    want += [O.list_directed_record([("r8", r[0]), ("r4", r[1]), ("r4", r[2])]) for r in dielf]
    assert open(path).read() == "\n".join(want) + "\n"
    back = _read_table(path, 1)                           # bseoptprop's list-directed read of the file
    assert np.array_equal(back[:, 0], dielf[:, 0])        # 17 significant digits: REAL(8) round-trips
    assert np.array_equal(back[:, 1:].astype(np.float32), dielf[:, 1:].astype(np.float32))

    nq, dim = 7, 5
    qpath = np.zeros((nq, 4))
    qpath[:, 0] = np.linspace(0.0, 1.0, nq)
    exk = np.sort(rng.uniform(1.5, 4.0, (dim, nq)), axis=0)
    path = os.path.join(tmp_path, "bands_bse.dat")
    api.write_bands_bse(path, qpath, exk)
    want = []
    for b in range(dim):
        want += [O.list_directed_record([("r4", qpath[i, 0]), ("r8", exk[b, i])]) for i in range(nq)] + [""]
    assert open(path).read() == "\n".join(want) + "\n"

    nk = 9
    kpt = rng.uniform(-0.5, 0.5, (nk, 3))
    act = rng.uniform(0, 5, (nk, 6))
    act[2, 5] = np.nan                                     # (sp - sm)/(sp + sm) of a k-point with no activity
    path = os.path.join(tmp_path, "dichroism.dat")
    api.write_bz_act(path, kpt, act[:, 5])
    want = [O.list_directed_record([("r4", k[0]), ("r4", k[1]), ("r4", k[2]), ("r8", a)])
            for k, a in zip(kpt, act[:, 5])]
    assert open(path).read() == "\n".join(want) + "\n"
    assert open(path).read().splitlines()[2].endswith("NaN")
