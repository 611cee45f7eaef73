"""Python mirror of the WTB exciton-path interface over the C ABI of libwtb_gb300.so.

The names and argument meanings follow the Fortran subroutines the library replaces
(``eigsys``, ``monhkhorst_pack``, ``bsesolver``, ``slepc_solver``, ``dielbsev``/``dielbsep``,
``bsedielraw``/``bsedielrawpol``, ``spoptics``, ``spdielraw``/``spdielrawpol``, ``bseoptprop``/``bseoptproppol``
and the ``module_coulomb`` potentials); arrays cross the boundary in
Fortran column-major order exactly as the Fortran caller would pass them.  There is no CPU
fallback: if the shared library is missing, importing this module raises.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from dataclasses import dataclass

import numpy as np

from .synthetic import BSEParams, TBSystem

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libwtb_gb300.so")

WTB_OK, WTB_EBADARG, WTB_ENOMEM, WTB_ENOCONV, WTB_ETIMEOUT, WTB_ENAN, WTB_ECUDA, WTB_ESTATE, WTB_ENODEV = range(9)
STATUS_NAMES = {0: "WTB_OK", 1: "WTB_EBADARG", 2: "WTB_ENOMEM", 3: "WTB_ENOCONV", 4: "WTB_ETIMEOUT",
                5: "WTB_ENAN", 6: "WTB_ECUDA", 7: "WTB_ESTATE", 8: "WTB_ENODEV"}
STATUS = {v: k for k, v in STATUS_NAMES.items()}
PREC = {"fp64": 0, "fp32": 1, "bf16x3": 2, "bf16x6": 3}
OPS = {"dense": 0, "matfree": 1}
COULTYPES = {"V2DK": 0, "V3D": 1, "V3DL": 2, "V2DT": 3, "V2DT2": 4, "V2DOH": 5, "V2DRK": 6, "V1DT": 7, "V0DT": 8}
COMPONENTS = ("xx", "yy", "zz", "xy", "xz", "yz", "sp", "sm")
POL_COMPONENTS = ("xx", "yy", "zz", "sp", "sm")
# the columns of spoptics' vecres records (src/module_bse.F90:4969-4990)
SP_COLUMNS = ("kx", "ky", "kz", "nocp", "ic", "iv", "energy", "xx", "yy", "zz", "xy", "xz", "yz", "sp", "sm")


class WTBError(RuntimeError):
    """A non-zero status from the library; ``code`` is the WTB_* status, the text is the reference's."""

    def __init__(self, code: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {message}")
        self.code = code


class CParams(C.Structure):
    _fields_ = [("ngrid", C.c_int * 3), ("nc", C.c_int), ("nv", C.c_int), ("mshift", C.c_double * 3),
                ("coultype", C.c_int), ("renorm", C.c_int), ("ktol", C.c_double), ("ediel", C.c_double * 3),
                ("ez", C.c_double), ("w_coul", C.c_double), ("r0", C.c_double), ("lc", C.c_double),
                ("cshift", C.c_double), ("ebse0", C.c_double), ("ebsef", C.c_double), ("numbse", C.c_int),
                ("nev", C.c_int), ("precision", C.c_int), ("op", C.c_int), ("tol", C.c_double),
                ("maxit", C.c_int), ("block", C.c_int)]


class CTempParams(C.Structure):
    _fields_ = [("temp", C.c_double), ("ta", C.c_int), ("st", C.c_double), ("phavg", C.c_double),
                ("dtfull", C.c_int), ("cpol", C.c_int)]


TEMP_GAP_CORRECTIONS = {"FA": 0, "VE": 1, "BE": 2}


class CSystem(C.Structure):
    _fields_ = [("w90basis", C.c_int), ("nvec", C.c_int), ("rvec", C.POINTER(C.c_int)), ("ffactor", C.POINTER(C.c_int)),
                ("hopmatrices", C.POINTER(C.c_double)), ("ihopmatrices", C.POINTER(C.c_double)),
                ("rlat", C.POINTER(C.c_double)), ("efermi", C.c_double), ("scs", C.c_double), ("systype_np", C.c_int)]


class CTimings(C.Structure):
    _fields_ = [("t_bands_ms", C.c_double), ("t_build_ms", C.c_double), ("t_solve_ms", C.c_double),
                ("t_optics_ms", C.c_double), ("t_total_ms", C.c_double), ("iterations", C.c_int),
                ("matvec_columns", C.c_int), ("max_rel_residual", C.c_double), ("refine_shift_max", C.c_double),
                ("kernel_launches", C.c_int)]


def _load():
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with __graft_entry__.build(); there is no CPU fallback")
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    sigs = {
        "wtb_ctx_create": [C.POINTER(P), C.c_int],
        "wtb_ctx_destroy": [P],
        "wtb_set_hr": [P, C.c_int, C.c_int, ip, ip, dp, dp, dp, C.c_double, C.c_double, C.c_int],
        "wtb_eigsys": [C.c_int, C.c_double, C.c_double, ip, ip, C.c_double, C.c_double, C.c_double, C.c_int,
                       C.c_int, dp, ip, dp, dp, C.c_double, dp, dp],
        "wtb_monhkhorst_pack": [C.c_int, C.c_int, C.c_int, dp, dp, dp, dp, dp],
        "wtb_eigsys_mesh": [P, C.c_int, dp, C.c_int, C.c_int, dp, dp, ip],
        "wtb_coulomb_table": [P, C.POINTER(CParams), C.c_int, dp, C.c_int, dp, dp],
        "wtb_optsp": [P, C.POINTER(CParams), dp],
        "wtb_bse_build": [P, C.POINTER(CParams), dp],
        "wtb_bse_matvec": [P, C.POINTER(CParams), C.c_int, dp, dp],
        "wtb_slepc_solver": [P, dp, dp, dp, C.c_int, C.c_int],
        "wtb_dielbse": [P, C.c_int, C.c_int, dp, dp, dp, C.c_int, dp],
        "wtb_bsesolver": [P, C.POINTER(CParams), dp, dp, dp, C.POINTER(CTimings)],
        "wtb_bsedielraw": [P, C.POINTER(CParams), C.c_int, dp, dp, dp],
        "wtb_bseoptprop": [P, C.c_int, dp, dp],
        "wtb_bsedielrawpol": [P, C.POINTER(CParams), C.c_int, dp, dp, dp],
        "wtb_spdielraw": [P, C.POINTER(CParams), C.c_int, dp, dp, dp],
        "wtb_spdielrawpol": [P, C.POINTER(CParams), C.c_int, dp, dp, dp],
        "wtb_bseoptproppol": [P, C.c_int, dp, dp],
        "wtb_spoptics": [P, C.POINTER(CParams), C.POINTER(C.c_float)],
        "wtb_spoptpolbz": [P, C.POINTER(CParams), dp],
        "wtb_kpathbse": [dp, dp, dp, C.c_int, dp, C.c_int, dp],
        "wtb_bse_build_q": [P, C.POINTER(CParams), dp, dp],
        "wtb_bsebnds": [P, C.POINTER(CParams), C.c_int, dp, dp],
        "wtb_zheev": [P, C.c_int, dp, C.c_int, dp],
        "wtb_zheev_vectors": [P, C.c_int, dp, C.c_int, dp, dp],
        "wtb_write_bse_opt_diel": [C.c_char_p, C.c_int, dp, dp, C.c_int],
        "wtb_write_sp_optics": [C.c_char_p, C.c_int, C.POINTER(C.c_float), C.c_int],
        "wtb_write_tm_coef": [C.c_char_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_int],
        "wtb_write_exc_wf": [C.c_char_p, C.c_int, C.c_int, C.c_int, ip, dp, dp, C.c_int, C.c_double, dp],
        "wtb_bse_q_eigenpairs": [P, C.POINTER(CParams), dp, C.c_int, C.c_int, dp, dp],
        "wtb_exciton_lifetime": [P, C.c_char_p, ip, C.c_int, dp, C.c_int, dp],
        "wtb_write_exciton_lifetime": [C.c_char_p, C.c_int, dp, dp, C.c_int],
        "wtb_write_diel": [C.c_char_p, C.c_int, dp],
        "wtb_write_bands_bse": [C.c_char_p, C.c_int, C.c_int, dp, dp],
        "wtb_write_bz_act": [C.c_char_p, C.c_int, dp, dp],
        "wtb_fortran_format": [C.c_char, C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_int],
        "wtb_bsesolvertemp": [P, C.POINTER(CParams), C.POINTER(CTempParams), dp, dp, dp, dp],
        "wtb_bsebndstemp": [P, C.POINTER(CParams), C.POINTER(CTempParams), C.c_int, dp, dp],
        "wtb_spoptics_temp": [P, C.POINTER(CParams), C.POINTER(CTempParams), C.POINTER(C.c_float)],
        "wtb_bse_backward": [P, C.POINTER(CParams), dp, dp, dp, dp, dp, C.POINTER(CTimings)],
        "wtb_spectrum_loss": [P, C.POINTER(CParams), C.c_int, C.c_int, dp, dp, dp, dp, dp, dp],
        "wtb_batch_create": [C.POINTER(P), C.c_int, C.c_int],
        "wtb_batch_destroy": [P],
        "wtb_batch_bsesolver": [P, C.c_int, C.POINTER(CSystem), C.POINTER(CParams), C.c_int, dp, dp, ip, ip, dp],
        "wtb_batch_matvec": [P, C.c_int, dp, dp],
        "wtb_batch_timings": [P, dp],
        "wtb_autotune_report": [C.c_char_p, C.c_int],
        "wtb_coulomb_pair": [C.POINTER(CParams), dp, dp, dp, dp],
        "wtb_hlm": [C.c_double, C.c_double, C.c_double, ip, C.c_int, C.c_int, dp, ip, dp, dp, dp, dp, dp],
        "wtb_optsp_pair": [C.c_double, dp, C.c_double, dp, C.c_double, C.c_double, C.c_double, ip, C.c_double,
                           C.c_int, C.c_int, dp, ip, dp, dp, dp, dp, dp],
        "wtb_optdiel": [C.c_int, C.c_double, C.c_int, ip, C.c_double, dp, dp, C.c_double, dp, dp],
        "wtb_operator_form": [P],
    }
    for name, args in sigs.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = C.c_int
    lib.wtb_batch_error.argtypes = [P, C.c_int]
    lib.wtb_batch_error.restype = C.c_char_p
    lib.wtb_last_error.argtypes = [P]
    lib.wtb_last_error.restype = C.c_char_p
    lib.wtb_version.restype = C.c_int
    lib.wtb_kernel_launch_count.restype = C.c_longlong
    lib.wtb_ctx_stream.argtypes = [P]
    lib.wtb_ctx_stream.restype = C.c_void_p
    lib.wtb_profile_enable.argtypes = [P, C.c_int]
    lib.wtb_profile_enable.restype = C.c_int
    lib.wtb_profile_read.argtypes = [P, dp, C.POINTER(C.c_longlong), dp, dp]
    lib.wtb_profile_read.restype = C.c_int
    return lib


_lib = _load()


def lib():
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int)) if a is not None else None


def _f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _c128(a):
    return np.asfortranarray(np.asarray(a, dtype=np.complex128))


def cparams(p: BSEParams, precision="fp64", op="dense", tol=0.0, maxit=0, block=0) -> CParams:
    c = CParams()
    for i in range(3):
        c.ngrid[i] = int(p.ngrid[i])
        c.mshift[i] = float(p.mshift[i])
        c.ediel[i] = float(p.ediel[i])
    c.nc, c.nv = int(p.nc), int(p.nv)
    c.coultype = COULTYPES[p.coultype] if isinstance(p.coultype, str) else int(p.coultype)
    c.renorm = 1 if p.renorm else 0
    c.ktol, c.ez, c.w_coul, c.r0, c.lc = float(p.ktol), float(p.ez), float(p.w_coul), float(p.r0), float(p.lc)
    c.cshift, c.ebse0, c.ebsef = float(p.cshift), float(p.ebse0), float(p.ebsef)
    c.numbse, c.nev = int(p.numbse), int(p.nev)
    c.precision = PREC[precision] if isinstance(precision, str) else int(precision)
    c.op = OPS[op] if isinstance(op, str) else int(op)
    c.tol, c.maxit, c.block = float(tol), int(maxit), int(block)
    return c


def autotune_report() -> dict:
    """The launch shapes chosen by the autotuner in this process (wtb_autotune_report): the source hash its
    cache is keyed by, the cache file, and one entry per (shape, parameter)."""
    n = _lib.wtb_autotune_report(None, 0)
    buf = C.create_string_buffer(n + 1)
    _lib.wtb_autotune_report(buf, n + 1)
    return json.loads(buf.value.decode())


OPERATOR_FORMS = ("none", "tensor-core split-BF16 product", "FP32 CUDA-core product", "FP64 CUDA-core product",
                  "FP32 FFT convolution")


def kernel_launch_count() -> int:
    return int(_lib.wtb_kernel_launch_count())


def monhkhorst_pack(n1, n2, n3, shift, rlat1, rlat2, rlat3):
    """monhkhorst_pack (src/module_kmesh.F90:338-386): returns kpt (n1*n2*n3, 3)."""
    kpt = np.zeros((n1 * n2 * n3, 3), order="F")
    r = _lib.wtb_monhkhorst_pack(n1, n2, n3, _dp(_f64(shift)), _dp(_f64(rlat1)), _dp(_f64(rlat2)),
                                 _dp(_f64(rlat3)), _dp(kpt))
    if r:
        raise WTBError(r, "monhkhorst_pack: bad arguments")
    return np.ascontiguousarray(kpt)


def kpathbse(rlat1, rlat2, rlat3, ks, npts):
    """kpathbse (src/module_kmesh.F90:124-193): ks (nks, 3) reduced corner points in (start, end) pairs; returns
    qpath ((nks//2)*npts, 4) = (path coordinate, Qx, Qy, Qz)."""
    ks = np.asfortranarray(np.asarray(ks, dtype=np.float64))
    nq = (ks.shape[0] // 2) * int(npts)
    q = np.zeros((nq, 4), order="F")
    r = _lib.wtb_kpathbse(_dp(_f64(rlat1)), _dp(_f64(rlat2)), _dp(_f64(rlat3)), ks.shape[0], _dp(ks), int(npts),
                          _dp(q))
    if r:
        raise WTBError(r, "kpathbse: bad arguments")
    return np.ascontiguousarray(q)


def fortran_format(kind, x, w, d):
    """One Fortran edit descriptor (F, E or I) as the output writers apply it; kind G with (w, d) = (25, 17) or
    (16, 9) is one REAL(8) or REAL(4) item of a list-directed record."""
    buf = C.create_string_buffer(w + 1)
    r = _lib.wtb_fortran_format(kind.encode(), float(x), int(w), int(d), buf, w + 1)
    if r:
        raise WTBError(r, "fortran_format: bad arguments")
    return buf.value.decode()


def _w(r, what):
    if r:
        raise WTBError(r, what + ": cannot write the file")


def write_bse_opt_diel(path, Ws, acts, pol=False):
    """bse_opt_diel.dat (pol=False) or bse_opt_diel-pol.dat from Ws (dim,) and acts {comp: (dim,)}."""
    Ws = np.ascontiguousarray(Ws, dtype=np.float64)
    A = np.zeros((len(Ws), 8), order="F")
    for i, c in enumerate(COMPONENTS):
        A[:, i] = acts[c]
    _w(_lib.wtb_write_bse_opt_diel(os.fsencode(path), len(Ws), _dp(Ws), _dp(A), int(bool(pol))),
       "wtb_write_bse_opt_diel")


def write_sp_optics(path, rec, pol=False):
    rec = np.asfortranarray(rec, dtype=np.float32)
    _w(_lib.wtb_write_sp_optics(os.fsencode(path), rec.shape[0], rec.ctypes.data_as(C.POINTER(C.c_float)),
                                int(bool(pol))), "wtb_write_sp_optics")


def write_tm_coef(path, nk, nc, nv, rec, pol=False):
    rec = np.asfortranarray(rec, dtype=np.float32)
    _w(_lib.wtb_write_tm_coef(os.fsencode(path), nk, nc, nv, rec.ctypes.data_as(C.POINTER(C.c_float)),
                              int(bool(pol))), "wtb_write_tm_coef")


def write_exc_wf(path, nocpk, kpt, nc, nv, excnum, energy, ewf, q4=None):
    """exc_wf_<n>.dat (excwf2), or with q4 (a Q-path row) exc_wf_<n>_<q>.dat (excwfi2)."""
    nocp = np.ascontiguousarray(nocpk, dtype=np.int32)
    k = np.asfortranarray(kpt, dtype=np.float64)
    e = np.ascontiguousarray(ewf, dtype=np.complex128)
    q = None if q4 is None else np.ascontiguousarray(q4, dtype=np.float64)
    _w(_lib.wtb_write_exc_wf(os.fsencode(path), len(nocp), nc, nv, nocp.ctypes.data_as(C.POINTER(C.c_int)), _dp(k),
                             _dp(q), int(excnum), float(energy), e.ctypes.data_as(C.POINTER(C.c_double))),
       "wtb_write_exc_wf")


def write_exciton_lifetime(path, energy, lft, pol=False):
    """exciton_lifetime.dat (lft (dim, 4)) or exciton_lifetime-pol.dat (pol=True, lft (dim, 6))."""
    e = np.ascontiguousarray(energy, dtype=np.float64)
    L = np.asfortranarray(lft, dtype=np.float64)
    assert L.shape == (len(e), 6 if pol else 4)
    _w(_lib.wtb_write_exciton_lifetime(os.fsencode(path), len(e), _dp(e), _dp(L), int(bool(pol))),
       "wtb_write_exciton_lifetime")


def write_diel(path, dielf):
    """One component of bse_diel_*.dat or sp_diel*.dat from dielf (numbse, 3) = omega, eps1, eps2 (one value of
    the dict bsedielraw / spdielraw return)."""
    D = np.asfortranarray(dielf, dtype=np.float64)
    assert D.ndim == 2 and D.shape[1] == 3
    _w(_lib.wtb_write_diel(os.fsencode(path), D.shape[0], _dp(D)), "wtb_write_diel")


def write_bands_bse(path, qpath, exk):
    """bands_bse.dat from qpath (nq, 4) (kpathbse) and exk (dim, nq) (bsebnds / bsebndstemp)."""
    q = np.asfortranarray(qpath, dtype=np.float64)
    E = np.asfortranarray(exk, dtype=np.float64)
    assert q.ndim == 2 and E.ndim == 2 and E.shape[1] == q.shape[0]
    _w(_lib.wtb_write_bands_bse(os.fsencode(path), q.shape[0], E.shape[0], _dp(q), _dp(E)), "wtb_write_bands_bse")


def write_bz_act(path, kpt, value):
    """One of bz_act_x/y/z/sp/sm.dat or dichroism.dat from kpt (nk, 3) and one column of spoptpolbz's act."""
    k = np.asfortranarray(kpt, dtype=np.float64)
    v = np.ascontiguousarray(value, dtype=np.float64)
    assert k.shape == (len(v), 3)
    _w(_lib.wtb_write_bz_act(os.fsencode(path), len(v), _dp(k), _dp(v)), "wtb_write_bz_act")


def eigsys(nthreads, scs, exc, nocp, ffactor, kx, ky, kz, w90basis, nvec, rlat, rvec, hopmatrices, ihopmatrices,
           efermi):
    """eigsys (src/module_hamiltonian.F90:200-320), same argument list; H(R) arrays with the reference's
    shapes: rvec (nvec,3), hopmatrices (nvec,w,w).  Returns (nocp, energias (w,), autovetores (w,w))."""
    n = C.c_int(int(nocp))
    en = np.zeros(w90basis)
    av = np.zeros((w90basis, w90basis), dtype=np.complex128, order="F")
    ff = np.asfortranarray(np.asarray(ffactor, dtype=np.int32))
    rv = np.asfortranarray(np.asarray(rvec, dtype=np.int32))
    r = _lib.wtb_eigsys(int(nthreads), float(scs), float(exc), C.byref(n), _ip(ff), float(kx), float(ky), float(kz),
                        int(w90basis), int(nvec), _dp(_f64(rlat)), _ip(rv), _dp(_f64(hopmatrices)),
                        _dp(_f64(ihopmatrices)), float(efermi), _dp(en), _dp(av))
    if r:
        raise WTBError(r, "eigsys failed")
    return n.value, en, av


def coulomb_pair(p: BSEParams, rlat, kpt1, kpt2) -> float:
    """One value of the potential p.coultype at (kpt1, kpt2) with the lattice rlat (rlat[i] = a_(i+1)), as the
    scalar functions of module_coulomb return it (v2drk, v3diel, ...; src/module_coulomb.F90:11-442)."""
    v = C.c_double()
    cp = cparams(p)
    r = _lib.wtb_coulomb_pair(C.byref(cp), _dp(_f64(rlat)), _dp(np.ascontiguousarray(kpt1, dtype=np.float64)),
                              _dp(np.ascontiguousarray(kpt2, dtype=np.float64)), C.byref(v))
    if r:
        raise WTBError(r, "wtb_coulomb_pair failed")
    return v.value


def _hr_args(sysm):
    return (_ip(np.asfortranarray(np.asarray(sysm.ffactor, dtype=np.int32))), int(sysm.w90basis), int(sysm.nvec),
            _dp(_f64(sysm.rlat)), _ip(np.asfortranarray(np.asarray(sysm.rvec, dtype=np.int32))),
            _dp(_f64(sysm.hop)), _dp(_f64(sysm.ihop)))


def hlm(k, sysm):
    """hlm (src/module_optics.F90:12-108) at one k-point: (hx, hy, hz), each (w, w) complex."""
    w = sysm.w90basis
    out = [np.zeros((w, w), dtype=np.complex128, order="F") for _ in range(3)]
    ff, w_, nv_, rl, rv, hp, ih = _hr_args(sysm)
    r = _lib.wtb_hlm(float(k[0]), float(k[1]), float(k[2]), ff, w_, nv_, rl, rv, hp, ih, *(_dp(o) for o in out))
    if r:
        raise WTBError(r, "wtb_hlm failed")
    return tuple(out)


def optsp_pair(ev, vv, ec, vc, k, sme, sysm):
    """optsp (src/module_optics.F90:113-167) for one (valence, conduction) pair: (hrx, hry, hrz)."""
    out = [np.zeros(1, dtype=np.complex128) for _ in range(3)]
    ff, w_, nv_, rl, rv, hp, ih = _hr_args(sysm)
    r = _lib.wtb_optsp_pair(float(ev), _dp(np.ascontiguousarray(vv, dtype=np.complex128)), float(ec),
                            _dp(np.ascontiguousarray(vc, dtype=np.complex128)), float(k[0]), float(k[1]), float(k[2]),
                            ff, float(sme), w_, nv_, rl, rv, hp, ih, *(_dp(o) for o in out))
    if r:
        raise WTBError(r, "wtb_optsp_pair failed")
    return tuple(complex(o[0]) for o in out)


def optdiel(rtype, vc, ngrid, elux, exciton, fosc, sme):
    """optdiel (src/module_optics.F90:171-255) at one photon energy: (rpart, ipart)."""
    E = np.ascontiguousarray(exciton, dtype=np.float64)
    f = np.ascontiguousarray(fosc, dtype=np.float64)
    g = np.ascontiguousarray(ngrid, dtype=np.int32)
    rp, ipart = C.c_double(), C.c_double()
    r = _lib.wtb_optdiel(int(rtype), float(vc), len(E), _ip(g), float(elux), _dp(E), _dp(f), float(sme), C.byref(rp),
                         C.byref(ipart))
    if r:
        raise WTBError(r, "wtb_optdiel failed")
    return rp.value, ipart.value


class Context:
    """One device context (``wtb_ctx``); owns device buffers and the stream."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        r = _lib.wtb_ctx_create(C.byref(h), int(device))
        if r:
            raise WTBError(r, "no usable CUDA device")
        self._h = h
        self.system: TBSystem | None = None

    def close(self):
        if self._h:
            _lib.wtb_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, r, what):
        if r:
            msg = _lib.wtb_last_error(self._h)
            raise WTBError(r, f"{what}: {msg.decode() if msg else ''}")

    # -------------------------------------------------------------------- module_hamiltonian globals
    def set_hr(self, s: TBSystem):
        rv = np.asfortranarray(s.rvec.astype(np.int32))
        ff = np.asfortranarray(s.ffactor.astype(np.int32))
        self._chk(_lib.wtb_set_hr(self._h, int(s.w90basis), int(s.nvec), _ip(rv), _ip(ff), _dp(_f64(s.hop)),
                                  _dp(_f64(s.ihop)), _dp(_f64(s.rlat)), float(s.efermi), float(s.scs),
                                  1 if s.systype == "NP" else 0), "wtb_set_hr")
        self.system = s

    def eigsys_mesh(self, kpt, nv, nc):
        """Band loop of bsesolver: returns eigv (nk, nv+nc), vector (nk, nv+nc, w), nocpk (nk,)."""
        kpt = np.asarray(kpt, dtype=np.float64)
        nk = kpt.shape[0]
        w = self.system.w90basis
        eigv = np.zeros((nk, nv + nc), order="F")
        vec = np.zeros((nk, nv + nc, w), dtype=np.complex128, order="F")
        nocp = np.zeros(nk, dtype=np.int32)
        self._chk(_lib.wtb_eigsys_mesh(self._h, nk, _dp(_f64(kpt)), int(nv), int(nc), _dp(eigv), _dp(vec), _ip(nocp)),
                  "wtb_eigsys_mesh")
        return np.ascontiguousarray(eigv), np.ascontiguousarray(vec), nocp

    def coulomb_table(self, p: BSEParams, kpt1, kpt2=None):
        kpt1 = np.asarray(kpt1, dtype=np.float64)
        kpt2 = kpt1 if kpt2 is None else np.asarray(kpt2, dtype=np.float64)
        V = np.zeros((len(kpt1), len(kpt2)), order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_coulomb_table(self._h, C.byref(cp), len(kpt1), _dp(_f64(kpt1)), len(kpt2),
                                         _dp(_f64(kpt2)), _dp(V)), "wtb_coulomb_table")
        return np.ascontiguousarray(V)

    def optsp(self, p: BSEParams):
        dim = p.dim
        hr = np.zeros((dim, 5), dtype=np.complex128, order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_optsp(self._h, C.byref(cp), _dp(hr)), "wtb_optsp")
        return hr.T.copy()

    def bse_build(self, p: BSEParams, precision="fp64"):
        dim = p.dim
        H = np.zeros((dim, dim), dtype=np.complex128, order="F")
        cp = cparams(p, precision=precision)
        self._chk(_lib.wtb_bse_build(self._h, C.byref(cp), _dp(H)), "wtb_bse_build")
        return H

    def bse_build_q(self, p: BSEParams, q4):
        """The finite-Q BSE matrix (matrizelbsekq) for one Q-path row q4 = (path coordinate, Qx, Qy, Qz)."""
        dim = p.dim
        H = np.zeros((dim, dim), dtype=np.complex128, order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_bse_build_q(self._h, C.byref(cp), _dp(_f64(q4)), _dp(H)), "wtb_bse_build_q")
        return H

    def bse_q_eigenpairs(self, p: BSEParams, q4, il=1, nvec=1):
        """All eigenvalues W of the finite-Q matrix and the eigenvectors il..il+nvec-1 (1-based) as Z (dim, nvec)."""
        W = np.zeros(p.dim)
        Z = np.zeros((p.dim, nvec), dtype=np.complex128, order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_bse_q_eigenpairs(self._h, C.byref(cp), _dp(_f64(q4)), int(il), int(nvec), _dp(W),
                                            Z.ctypes.data_as(C.POINTER(C.c_double))), "wtb_bse_q_eigenpairs")
        return W, Z

    def bsebnds(self, p: BSEParams, qpath):
        """bsebnds: all finite-Q exciton energies, exk (dim, nq), for the rows of qpath."""
        qpath = np.asfortranarray(np.asarray(qpath, dtype=np.float64))
        nq = qpath.shape[0]
        exk = np.zeros((p.dim, nq), order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_bsebnds(self._h, C.byref(cp), nq, _dp(qpath), _dp(exk)), "wtb_bsebnds")
        return exk

    def bsebndstemp(self, p: BSEParams, qpath, temp, ta="FA", st=0.0, phavg=0.0):
        """bsebndstemp: all finite-Q exciton energies at temperature temp, exk (dim, nq)."""
        qpath = np.asfortranarray(np.asarray(qpath, dtype=np.float64))
        nq = qpath.shape[0]
        exk = np.zeros((p.dim, nq), order="F")
        tp = CTempParams(float(temp), TEMP_GAP_CORRECTIONS[ta] if isinstance(ta, str) else int(ta), float(st),
                         float(phavg), 1, 1)
        cp = cparams(p)
        self._chk(_lib.wtb_bsebndstemp(self._h, C.byref(cp), C.byref(tp), nq, _dp(qpath), _dp(exk)),
                  "wtb_bsebndstemp")
        return exk

    def zheev(self, A):
        """ZHEEV('N', 'U'): all eigenvalues (ascending) of the Hermitian matrix held in A's upper triangle."""
        A = np.asfortranarray(np.asarray(A, dtype=np.complex128))
        n = A.shape[0]
        W = np.zeros(n)
        self._chk(_lib.wtb_zheev(self._h, n, A.ctypes.data_as(C.POINTER(C.c_double)), n, _dp(W)), "wtb_zheev")
        return W

    def zheev_vectors(self, A):
        """ZHEEV('V', 'U'): (W ascending, Z (n, n) eigenvectors in columns) of the matrix in A's upper triangle."""
        A = np.asfortranarray(np.asarray(A, dtype=np.complex128))
        n = A.shape[0]
        W = np.zeros(n)
        Z = np.zeros((n, n), dtype=np.complex128, order="F")
        self._chk(_lib.wtb_zheev_vectors(self._h, n, A.ctypes.data_as(C.POINTER(C.c_double)), n, _dp(W),
                                         Z.ctypes.data_as(C.POINTER(C.c_double))), "wtb_zheev_vectors")
        return W, Z

    def bsesolvertemp(self, p: BSEParams, temp, ta="FA", st=0.0, phavg=0.0, dtfull=True, cpol=True,
                      want_vectors=False):
        """bsesolvertemp: all dim exciton energies Ws, the activities {comp: (dim,)}, fdeh, and (optionally) HE."""
        dim = p.dim
        Ws = np.zeros(dim)
        acts = np.zeros((dim, 8), order="F")
        f = np.zeros(dim)
        HE = np.zeros((dim, dim), dtype=np.complex128, order="F") if want_vectors else None
        tp = CTempParams(float(temp), TEMP_GAP_CORRECTIONS[ta] if isinstance(ta, str) else int(ta), float(st),
                         float(phavg), int(bool(dtfull)), int(bool(cpol)))
        cp = cparams(p)
        self._chk(_lib.wtb_bsesolvertemp(self._h, C.byref(cp), C.byref(tp), _dp(Ws), _dp(acts),
                                         None if HE is None else HE.ctypes.data_as(C.POINTER(C.c_double)),
                                         _dp(f)), "wtb_bsesolvertemp")
        out = {"Ws": Ws, "acts": {c: acts[:, i].copy() for i, c in enumerate(COMPONENTS)}, "fdeh": f}
        if want_vectors:
            out["HE"] = HE
        return out

    def exciton_lifetime(self, sysdim, ngrid, fosc, pol=False):
        """exclft over the rows fosc (dim, 7) of bse_opt_diel.dat: lft (dim, 4) for xx+yy+zz, xx, yy, zz; with
        pol the rows (dim, 6) of bse_opt_diel-pol.dat and lft (dim, 6) adding sp, sm (lifetimepol)."""
        F = np.asfortranarray(fosc, dtype=np.float64)
        assert F.shape[1] == (6 if pol else 7)
        g = np.ascontiguousarray(ngrid, dtype=np.int32)
        L = np.zeros((F.shape[0], 6 if pol else 4), order="F")
        self._chk(_lib.wtb_exciton_lifetime(self._h, sysdim.encode(), g.ctypes.data_as(C.POINTER(C.c_int)),
                                            F.shape[0], _dp(F), int(bool(pol)), _dp(L)), "wtb_exciton_lifetime")
        return L

    def operator_form(self) -> str:
        """The contraction form of the last BSE operator (wtb_operator_form)."""
        return OPERATOR_FORMS[int(_lib.wtb_operator_form(self._h))]

    def bse_matvec(self, p: BSEParams, X, precision="fp64", op="matfree"):
        """Y = H X for the bands of the last set-up (X: dim x ncol complex)."""
        X = _c128(X)
        if X.ndim == 1:
            X = X.reshape(-1, 1, order="F")
        Y = np.zeros_like(X, order="F")
        cp = cparams(p, precision=precision, op=op)
        self._chk(_lib.wtb_bse_matvec(self._h, C.byref(cp), X.shape[1], _dp(X), _dp(Y)), "wtb_bse_matvec")
        return Y

    def slepc_solver(self, HX, NE):
        HX = _c128(HX)
        NX = HX.shape[0]
        EX = np.zeros(NE)
        HE = np.zeros((NX, NE), dtype=np.complex128, order="F")
        self._chk(_lib.wtb_slepc_solver(self._h, _dp(HX), _dp(EX), _dp(HE), NX, NE), "wtb_slepc_solver")
        return EX, HE

    def dielbse(self, dimse, dimse1, excitonvec, hopt1, hopt2=None):
        A = _c128(excitonvec)[:, :dimse1]
        A = np.asfortranarray(A)
        h1 = _c128(hopt1)
        h2 = _c128(hopt2) if hopt2 is not None else None
        act = np.zeros(dimse)
        self._chk(_lib.wtb_dielbse(self._h, dimse, dimse1, _dp(A), _dp(h1), _dp(h2), 1 if h2 is not None else 0,
                                   _dp(act)), "wtb_dielbse")
        return act

    def bsesolver(self, p: BSEParams, precision="fp64", op="dense", tol=0.0, maxit=0, block=0,
                  want_vectors=False, out=None):
        """The bsesolver path; returns dict with Ws (dim,), acts {comp: (dim,)}, E (nev,), timings, HE.
        out: optional caller-owned output arrays {"Ws": (dim,), "acts": (dim, 8) Fortran order, "HE": (dim, nev)
        complex128 Fortran order} (e.g. page-locked memory, which the device copies into directly)."""
        dim = p.dim
        if out is not None:
            Ws, acts = out["Ws"], out["acts"]
            HE = out.get("HE") if want_vectors else None
            assert Ws.dtype == np.float64 and Ws.shape == (dim,) and Ws.flags.c_contiguous
            assert acts.dtype == np.float64 and acts.shape == (dim, 8) and acts.flags.f_contiguous
            assert HE is None or (HE.dtype == np.complex128 and HE.shape == (dim, p.nev) and HE.flags.f_contiguous)
        else:
            Ws = np.zeros(dim)
            acts = np.zeros((dim, 8), order="F")
            HE = np.zeros((dim, p.nev), dtype=np.complex128, order="F") if want_vectors else None
        t = CTimings()
        cp = cparams(p, precision=precision, op=op, tol=tol, maxit=maxit, block=block)
        self._chk(_lib.wtb_bsesolver(self._h, C.byref(cp), _dp(Ws), _dp(acts),
                                     None if HE is None else HE.ctypes.data_as(C.POINTER(C.c_double)), C.byref(t)),
                  "wtb_bsesolver")
        out = {"Ws": Ws, "E": Ws[: p.nev].copy(), "acts": {c: acts[:, i].copy() for i, c in enumerate(COMPONENTS)},
               "timings": {f: getattr(t, f) for f, _ in CTimings._fields_}}
        if want_vectors:
            out["HE"] = HE
        return out

    def bse_backward(self, p: BSEParams, dL_dE=None, dL_dfxx=None, precision="fp64"):
        """Gradient of L(E, f_xx) through the last bsesolver call (same p and precision): returns dict with
        dhop, dihop (nvec, w, w), dr0 and the timings.  dL_dE / dL_dfxx: (nev,) or None (zero)."""
        s = self.system
        dh = np.zeros((s.nvec, s.w90basis, s.w90basis), order="F")
        di = np.zeros_like(dh, order="F")
        dr0 = C.c_double(0.0)
        t = CTimings()
        cp = cparams(p, precision=precision, op="matfree")
        a = None if dL_dE is None else np.ascontiguousarray(dL_dE, dtype=np.float64)
        b = None if dL_dfxx is None else np.ascontiguousarray(dL_dfxx, dtype=np.float64)
        self._chk(_lib.wtb_bse_backward(self._h, C.byref(cp), _dp(a), _dp(b), _dp(dh), _dp(di),
                                        C.cast(C.byref(dr0), C.POINTER(C.c_double)), C.byref(t)),
                  "wtb_bse_backward")
        return {"dhop": np.array(dh), "dihop": np.array(di), "dr0": dr0.value,
                "timings": {f: getattr(t, f) for f, _ in CTimings._fields_}}

    def spectrum_loss(self, p: BSEParams, dimse, E, fxx, target):
        """L = sum_j (spinf eps2_xx(omega_j) - target_j)^2 and its cotangents (dL/dE, dL/dfxx)."""
        E = np.ascontiguousarray(E, dtype=np.float64)
        f = np.ascontiguousarray(fxx, dtype=np.float64)
        tg = np.ascontiguousarray(target, dtype=np.float64)
        nev = len(E)
        L = C.c_double(0.0)
        gE = np.zeros(nev)
        gf = np.zeros(nev)
        cp = cparams(p)
        self._chk(_lib.wtb_spectrum_loss(self._h, C.byref(cp), int(dimse), nev, _dp(E), _dp(f), _dp(tg),
                                         C.cast(C.byref(L), C.POINTER(C.c_double)), _dp(gE), _dp(gf)),
                  "wtb_spectrum_loss")
        return L.value, gE, gf

    def _dielraw(self, fn, name, p: BSEParams, Ws, acts, comps):
        Ws = np.asarray(Ws, dtype=np.float64)
        dimse = len(Ws)
        nc = len(comps)
        A = np.zeros((dimse, nc), order="F")
        for i, cname in enumerate(comps):
            A[:, i] = acts[cname]
        dielf = np.zeros((p.numbse, 3, nc), order="F")
        cp = cparams(p)
        self._chk(fn(self._h, C.byref(cp), dimse, _dp(_f64(Ws)), _dp(A), _dp(dielf)), name)
        return {cname: dielf[:, :, i].copy() for i, cname in enumerate(comps)}

    def bsedielraw(self, p: BSEParams, Ws, acts):
        """Returns dict comp -> (numbse, 3) [omega, eps1, eps2] for xx yy zz xy xz yz."""
        return self._dielraw(_lib.wtb_bsedielraw, "wtb_bsedielraw", p, Ws, acts, COMPONENTS[:6])

    def bsedielrawpol(self, p: BSEParams, Ws, acts):
        """bsedielrawpol: dict comp -> (numbse, 3) for xx yy zz sp sm (acts: dict with those keys)."""
        return self._dielraw(_lib.wtb_bsedielrawpol, "wtb_bsedielrawpol", p, Ws, acts, POL_COMPONENTS)

    def spdielraw(self, p: BSEParams, esp, acts):
        """spdielraw: the independent-particle spectrum of the transitions esp, acts xx yy zz xy xz yz."""
        return self._dielraw(_lib.wtb_spdielraw, "wtb_spdielraw", p, esp, acts, COMPONENTS[:6])

    def spdielrawpol(self, p: BSEParams, esp, acts):
        """spdielrawpol: the independent-particle spectrum for xx yy zz sp sm."""
        return self._dielraw(_lib.wtb_spdielrawpol, "wtb_spdielrawpol", p, esp, acts, POL_COMPONENTS)

    def spoptics_temp(self, p: BSEParams, temp, ta="FA", st=0.0, phavg=0.0):
        """bsesolvertemp's IPA records: spoptics with scs + tcor and f-weighted activity columns."""
        dim = p.ngrid[0] * p.ngrid[1] * p.ngrid[2] * p.nc * p.nv
        rec = np.zeros((dim, 15), dtype=np.float32, order="F")
        tp = CTempParams(float(temp), TEMP_GAP_CORRECTIONS[ta] if isinstance(ta, str) else int(ta), float(st),
                         float(phavg), 1, 1)
        cp = cparams(p)
        self._chk(_lib.wtb_spoptics_temp(self._h, C.byref(cp), C.byref(tp), rec.ctypes.data_as(C.POINTER(C.c_float))),
                  "wtb_spoptics_temp")
        return rec

    def spoptpolbz(self, p: BSEParams):
        """spoptpolbz: act (nk, 6) = x y z sp sm activity per k-point of the mesh and the dichroism."""
        nk = p.ngrid[0] * p.ngrid[1] * p.ngrid[2]
        act = np.zeros((nk, 6), order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_spoptpolbz(self._h, C.byref(cp), _dp(act)), "wtb_spoptpolbz")
        return act

    def spoptics(self, p: BSEParams):
        """spoptics: the (dimsp, 15) float32 records (columns SP_COLUMNS) sorted by transition energy."""
        dim = p.ngrid[0] * p.ngrid[1] * p.ngrid[2] * p.nc * p.nv
        rec = np.zeros((dim, 15), dtype=np.float32, order="F")
        cp = cparams(p)
        self._chk(_lib.wtb_spoptics(self._h, C.byref(cp), rec.ctypes.data_as(C.POINTER(C.c_float))),
                  "wtb_spoptics")
        return rec

    def _optprop(self, fn, name, dielf: dict, comps):
        n = next(iter(dielf.values())).shape[0]
        nc = len(comps)
        D = np.zeros((n, 3, nc), order="F")
        for i, cname in enumerate(comps):
            D[:, :, i] = dielf[cname]
        props = np.zeros((n, nc, 5), order="F")
        self._chk(fn(self._h, n, _dp(D), _dp(props)), name)
        names = ("refr", "ext", "refl", "abs", "eloss")
        return {nm: {cname: props[:, i, q].copy() for i, cname in enumerate(comps)}
                for q, nm in enumerate(names)}

    def bseoptprop(self, dielf: dict):
        return self._optprop(_lib.wtb_bseoptprop, "wtb_bseoptprop", dielf, COMPONENTS[:6])

    def bseoptproppol(self, dielf: dict):
        """bseoptproppol / spoptproppol: the optical constants of an xx yy zz sp sm spectrum."""
        return self._optprop(_lib.wtb_bseoptproppol, "wtb_bseoptproppol", dielf, POL_COMPONENTS)


class Batch:
    """Independent systems solved together on one device (``wtb_batch_*``): the split-BF16 forms as one joint
    eigensolve in one graph launch, other forms system by system."""

    def __init__(self, device: int = 0, nworkers: int = 1):
        h = C.c_void_p()
        r = _lib.wtb_batch_create(C.byref(h), int(device), int(nworkers))
        if r:
            raise WTBError(r, "wtb_batch_create failed")
        self._h = h

    def close(self):
        if self._h:
            _lib.wtb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bsesolver(self, items, precision="bf16x3", op="matfree", tol=0.0, maxit=0, raise_on_error=True):
        """items: list of (TBSystem, BSEParams).  Returns (list of dicts {E, acts, status, error, iterations},
        host wall ms of the batch)."""
        n = len(items)
        nev_stride = max(p.nev for _, p in items) if n else 1
        keep = []
        systems = (CSystem * max(n, 1))()
        params = (CParams * max(n, 1))()
        for i, (s, p) in enumerate(items):
            arrs = (np.asfortranarray(s.rvec.astype(np.int32)), np.asfortranarray(s.ffactor.astype(np.int32)),
                    _f64(s.hop), _f64(s.ihop), _f64(s.rlat))
            keep.append(arrs)
            systems[i] = CSystem(int(s.w90basis), int(s.nvec), _ip(arrs[0]), _ip(arrs[1]), _dp(arrs[2]), _dp(arrs[3]),
                                 _dp(arrs[4]), float(s.efermi), float(s.scs), 1 if s.systype == "NP" else 0)
            params[i] = cparams(p, precision=precision, op=op, tol=tol, maxit=maxit)
        E = np.zeros((n, nev_stride))
        acts = np.zeros((n, 8, nev_stride))
        status = np.zeros(n, dtype=np.int32)
        iters = np.zeros(n, dtype=np.int32)
        wall = np.zeros(1)
        r = _lib.wtb_batch_bsesolver(self._h, n, systems, params, nev_stride, _dp(E), _dp(acts), _ip(status),
                                     _ip(iters), _dp(wall))
        out = []
        for i, (_, p) in enumerate(items):
            err = _lib.wtb_batch_error(self._h, i)
            out.append({"E": E[i, :p.nev].copy(),
                        "acts": {c: acts[i, a, :p.nev].copy() for a, c in enumerate(COMPONENTS)},
                        "status": int(status[i]), "error": err.decode() if err else "", "iterations": int(iters[i])})
        if r and raise_on_error:
            bad = next(i for i in range(n) if status[i])
            raise WTBError(int(r), f"wtb_batch_bsesolver: system {bad}: {out[bad]['error']}")
        return out, float(wall[0])

    def timings(self):
        """Times (ms) of the last joint batch call: host stage, build, run, collect; device set-up, solve and
        oscillator phases."""
        t = np.zeros(7)
        _lib.wtb_batch_timings(self._h, _dp(t))
        return dict(zip(("stage", "build", "run", "collect", "dev_setup", "dev_solve", "dev_oscillators"), t.tolist()))

    def matvec(self, Xs):
        """The joint operator of the last ``bsesolver`` call applied to one block per system: Xs[i] is
        (dim_i, ncol) complex; returns the list of H_i X_i."""
        ncol = Xs[0].shape[1]
        X = np.concatenate([np.asfortranarray(x, dtype=np.complex128).reshape(-1, order="F") for x in Xs])
        Y = np.zeros_like(X)
        r = _lib.wtb_batch_matvec(self._h, int(ncol), _dp(X), _dp(Y))
        if r:
            raise WTBError(r, "wtb_batch_matvec failed")
        out, off = [], 0
        for x in Xs:
            n = x.shape[0] * ncol
            out.append(Y[off:off + n].reshape(x.shape[0], ncol, order="F"))
            off += n
        return out
