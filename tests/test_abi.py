"""The C-ABI library: loads without a GPU and exports every entry point include/wtb_gpu.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "wtb_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[a-z_ ]+\**\s*\**(wtb_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("wtb_ctx_create", "wtb_set_hr", "wtb_eigsys", "wtb_bsesolver", "wtb_slepc_solver", "wtb_bsedielraw",
              "wtb_bseoptprop", "wtb_bse_build", "wtb_coulomb_table", "wtb_dielbse", "wtb_monhkhorst_pack"):
        assert n in names


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(os.path.join(ROOT, "wtb_gb300", "libwtb_gb300.so"))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_host_only_entry_points(built):
    """monhkhorst_pack is host arithmetic: matches the package's mesh without a GPU."""
    import numpy as np

    from wtb_gb300 import api, synthetic

    rlat = synthetic.hex_lattice()
    k = api.monhkhorst_pack(5, 4, 1, [0.1, 0.0, 0.0], rlat[0], rlat[1], rlat[2])
    ref = synthetic.monkhorst_pack((5, 4, 1), rlat, (0.1, 0.0, 0.0))
    np.testing.assert_allclose(k, ref, rtol=0, atol=1e-14)
    # against the oracle's restatement of monhkhorst_pack/recvec (single-precision pi): bit for bit
    from oracle import wtb_oracle as O

    for ng, shift in (((5, 4, 1), (0.1, 0.0, 0.0)), ((60, 60, 1), (0.0, 0.0, 0.0)), ((16, 16, 16), (0.0, 0.0, 0.0)),
                      ((7, 3, 2), (0.25, 0.5, 0.125))):
        k = api.monhkhorst_pack(ng[0], ng[1], ng[2], list(shift), rlat[0], rlat[1], rlat[2])
        np.testing.assert_array_equal(k, O.monhkhorst_pack(ng[0], ng[1], ng[2], shift, rlat))


def test_kpathbse_host_entry_matches_oracle(built):
    """kpathbse is host arithmetic: the library's Q path equals the oracle's bit for bit."""
    import numpy as np

    from oracle import wtb_oracle as O
    from wtb_gb300 import api, synthetic

    rlat = synthetic.hex_lattice()
    ks = np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0], [0.5, 0.0, 0.0], [1 / 3, 1 / 3, 0.0], [1 / 3, 1 / 3, 0.0],
                   [0.0, 0.0, 0.0]])
    q = api.kpathbse(rlat[0], rlat[1], rlat[2], ks, 7)
    ref = O.kpathbse(rlat, ks, 7)
    assert q.shape == ref.shape == (21, 4)
    assert np.array_equal(q, ref)


def test_no_device_is_an_error_not_a_fallback(built):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from wtb_gb300 import api

    with pytest.raises(api.WTBError) as e:
        api.Context(0)
    assert e.value.code == api.WTB_ENODEV
