"""The allocation-free oscillator-strength entry point (wtb_dielbse_noalloc).

It serves callers that cannot allocate device memory -- their device memory belongs to another allocator,
or they must not pay cudaMalloc's implicit synchronisation -- by keeping its partial sums in a fixed
device array.  Checked against wtb_dielbse (which allocates through its context) on two calls in a
row, so a second call that reads stale contents of the shared array would fail.  This file runs last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _entry():
    from wtb_gb300 import api

    f = api.lib().wtb_dielbse_noalloc
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p, ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _device_complex(torch, a):
    """Caller-owned device copy of a complex array in Fortran order (interleaved re/im doubles)."""
    flat = np.asfortranarray(a).ravel(order="F")
    return torch.from_numpy(flat.view(np.float64).copy()).cuda()


def test_noalloc_matches_dielbse_on_consecutive_calls(built):
    torch = pytest.importorskip("torch")
    from wtb_gb300 import api

    f = _entry()
    ctx = api.Context(0)
    rng = np.random.default_rng(21)
    # the second call changes the geometry (partial-sum blocks per row and rows), so a final kernel that read
    # slots the current call did not write would see the first call's stale sums
    for dimse, dimse1, pair in ((3100, 12, 1), (1500, 20, 0)):
        A = rng.normal(size=(dimse, dimse1)) + 1j * rng.normal(size=(dimse, dimse1))
        h1 = rng.normal(size=dimse) + 1j * rng.normal(size=dimse)
        h2 = rng.normal(size=dimse) + 1j * rng.normal(size=dimse)
        ref = ctx.dielbse(dimse, dimse1, A, h1, h2 if pair else None)
        dA, d1, d2 = _device_complex(torch, A), _device_complex(torch, h1), _device_complex(torch, h2)
        out = torch.full((dimse,), 7.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        free0 = torch.cuda.mem_get_info()[0]
        launches0 = api.kernel_launch_count()
        rc = f(dimse, dimse1, dA.data_ptr(), d1.data_ptr(), d2.data_ptr() if pair else None, pair, out.data_ptr(),
               None)
        torch.cuda.synchronize()
        assert rc == api.WTB_OK
        # the call allocates nothing on the device (its first call may load the module, hence from the second
        # call on) and launches its two kernels
        if pair == 0:
            assert torch.cuda.mem_get_info()[0] == free0
        assert api.kernel_launch_count() - launches0 == 2
        np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-12, atol=1e-14)
    ctx.close()


def test_noalloc_rejects_sizes_beyond_the_fixed_scratch(built):
    from wtb_gb300 import api

    f = _entry()
    dimse = 1024 * 300
    # the size check comes before any device access, so dummy non-null pointers are never touched
    rc = f(dimse, 300, 16, 16, None, 0, 16, None)
    assert rc == api.WTB_EBADARG
