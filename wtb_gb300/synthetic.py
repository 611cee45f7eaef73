"""Seeded synthetic tight-binding systems and BSE run parameters.

These are the inputs of the exciton path: a Wannier-style H(R) with the layout the reference's
``hamiltonian_input_read`` fills (``src/module_hamiltonian.F90:8-31``), plus the run keys that
``bsesolver`` and ``bsedielraw`` consume (``src/module_bse.F90:2023-2026``, ``:835``).

Recipe (shared by the GPU path, the tests and the benchmark):

* lattices: 2D hexagonal a = 3.2 A with a 20 A vacuum axis, or simple cubic a = 5 A;
* R sets: every lattice vector with Euclidean length <= rmax * a (37 vectors for the hexagonal
  lattice at rmax = 3, 33 for the cubic lattice at rmax = 2), ndegen = 1;
* H(R): Re and Im i.i.d. N(0, 1/2) * exp(-|R|/a) eV; one of each +-R pair is drawn and
  H(-R) = H(R)^H, H(0) = (X + X^H)/2;
* gap: -D/2 on the on-site energies of the first w/2 orbitals and +D/2 on the rest, with D
  bisected until the global gap over the run's k-mesh equals the target; the Fermi level sits
  mid-gap, so w/2 bands are occupied at every k.

No public dataset is involved; everything is drawn from ``numpy.random.default_rng(seed)``.
"""
from __future__ import annotations

import dataclasses
from dataclasses import dataclass, field

import numpy as np

PI_F32 = 3.1415927410125732  # acos(-1.) in default (single) precision, src/module_kmesh.F90:392


@dataclass
class TBSystem:
    """Module globals of ``module_hamiltonian`` (``src/module_hamiltonian.F90:5-16``).

    ``hop[iR, m, n]`` / ``ihop[iR, m, n]`` hold Re/Im H_mn(R); ``rvec[iR]`` are integer lattice
    coordinates; ``rlat[i]`` is lattice vector a_(i+1) in Angstrom (the reference's ``rlat(i,:)``).
    """

    w90basis: int
    rvec: np.ndarray          # (nvec, 3) int32
    ffactor: np.ndarray       # (nvec,) int32 (ndegen)
    hop: np.ndarray           # (nvec, w, w) float64
    ihop: np.ndarray          # (nvec, w, w) float64
    rlat: np.ndarray          # (3, 3) float64, row i = a_(i+1)
    efermi: float = 0.0
    scs: float = 0.0
    systype: str = "2D"

    @property
    def nvec(self) -> int:
        return int(self.rvec.shape[0])

    def copy(self) -> "TBSystem":
        return dataclasses.replace(self, rvec=self.rvec.copy(), ffactor=self.ffactor.copy(),
                                   hop=self.hop.copy(), ihop=self.ihop.copy(), rlat=self.rlat.copy())


@dataclass
class BSEParams:
    """Run keys of the exciton path (``src/module_input.F90:54-122`` defaults, ``:125-279`` keys).

    ``ediel`` = (EDIEL_T, EDIEL, EDIEL_B); ``ez`` = EDIEL_Z; ``w_coul`` = W_COUL; ``r0`` = R_0;
    ``lc`` = LC; ``ktol`` = KTOL; ``cshift`` = CSHIFT (both the optics denominator and the
    Lorentzian width, ``src/main.F90:106-109,184``); ``ebse0/ebsef/numbse`` = ENSPECI/ENSPECF/NESPEC;
    ``renorm`` = RNMD; ``nev`` = number of excitons (the reference hard-codes 100 at
    ``src/module_bse.F90:2432``).
    """

    ngrid: tuple = (1, 1, 1)
    nc: int = 1
    nv: int = 1
    mshift: tuple = (0.0, 0.0, 0.0)
    coultype: str = "V2DRK"
    ktol: float = 0.001
    ediel: tuple = (1.0, 1.0, 1.0)
    ez: float = 1.0
    w_coul: float = 0.0
    r0: float = 1.0
    lc: float = 1.0
    cshift: float = 0.01
    ebse0: float = 0.0
    ebsef: float = 3.0
    numbse: int = 6001
    nev: int = 100
    renorm: bool = True

    @property
    def nk(self) -> int:
        return int(self.ngrid[0] * self.ngrid[1] * self.ngrid[2])

    @property
    def dim(self) -> int:
        return self.nk * self.nc * self.nv


def hex_lattice(a: float = 3.2, c: float = 20.0) -> np.ndarray:
    return np.array([[a, 0.0, 0.0], [-0.5 * a, 0.5 * np.sqrt(3.0) * a, 0.0], [0.0, 0.0, c]])


def cubic_lattice(a: float = 5.0) -> np.ndarray:
    return np.eye(3) * a


def lattice_vectors(rlat: np.ndarray, rmax: float, dims: int) -> np.ndarray:
    """Integer R with |R_cart| <= rmax (Angstrom), sorted by length then lexicographically."""
    nmax = int(np.ceil(rmax / min(np.linalg.norm(rlat[i]) for i in range(dims)))) + 2
    rng1 = range(-nmax, nmax + 1)
    out = []
    for n1 in rng1:
        for n2 in rng1:
            for n3 in (rng1 if dims == 3 else [0]):
                R = np.array([n1, n2, n3])
                L = np.linalg.norm(R @ rlat)
                if L <= rmax + 1e-9:
                    out.append((round(L, 9), n1, n2, n3))
    out.sort()
    return np.array([[o[1], o[2], o[3]] for o in out], dtype=np.int32)


def random_hr(rng: np.random.Generator, w: int, rvec: np.ndarray, rlat: np.ndarray, a: float):
    """Hermitian-consistent random H(R): H(-R) = H(R)^H, H(0) Hermitian."""
    nR = rvec.shape[0]
    H = np.zeros((nR, w, w), dtype=np.complex128)
    index = {tuple(r): i for i, r in enumerate(rvec.tolist())}
    done = set()
    for i, r in enumerate(rvec.tolist()):
        if i in done:
            continue
        L = np.linalg.norm(np.asarray(r) @ rlat)
        scale = np.exp(-L / a)
        X = (rng.normal(0.0, np.sqrt(0.5), (w, w)) + 1j * rng.normal(0.0, np.sqrt(0.5), (w, w))) * scale
        j = index[tuple(-x for x in r)]
        if j == i:
            H[i] = 0.5 * (X + X.conj().T)
        else:
            H[i] = X
            H[j] = X.conj().T
        done.add(i)
        done.add(j)
    return H


def monkhorst_pack(ngrid, rlat, mshift=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Gamma-anchored mesh, k outer index i then j then l (``src/module_kmesh.F90:338-386``)."""
    a1, a2, a3 = rlat
    v23, v31, v12 = np.cross(a2, a3), np.cross(a3, a1), np.cross(a1, a2)
    vol = abs(a1 @ v23)
    f = (2.0 * PI_F32) / vol
    b1, b2, b3 = f * v23, f * v31, f * v12
    n1, n2, n3 = ngrid
    ks = b1 * mshift[0] + b2 * mshift[1] + b3 * mshift[2]
    kpt = np.empty((n1 * n2 * n3, 3))
    c = 0
    for i in range(n1):
        for j in range(n2):
            for l in range(n3):
                kpt[c] = (b1 / n1) * i + (b2 / n2) * j + (b3 / n3) * l + ks
                c += 1
    return kpt


def bands_on_mesh(hop_c: np.ndarray, rvec: np.ndarray, rlat: np.ndarray, kpt: np.ndarray) -> np.ndarray:
    """All band energies (Nk, w) of H(k) = sum_R e^{ik.R} H(R), without the Fermi shift."""
    Rc = rvec @ rlat
    ph = np.exp(1j * (kpt @ Rc.T))                     # (Nk, nR)
    w = hop_c.shape[1]
    Hk = (ph @ hop_c.reshape(len(rvec), w * w)).reshape(-1, w, w)
    Hk = 0.5 * (Hk + np.conj(np.transpose(Hk, (0, 2, 1))))
    return np.linalg.eigvalsh(Hk)


def set_gap(hop_c: np.ndarray, rvec: np.ndarray, rlat: np.ndarray, kpt: np.ndarray, gap: float):
    """Bisect the on-site split D so the global gap between bands w/2 and w/2+1 equals ``gap``.

    Returns (H(R) with the split applied, efermi at mid-gap, smallest band spacing seen)."""
    w = hop_c.shape[1]
    i0 = int(np.flatnonzero(np.all(rvec == 0, axis=1))[0])
    split = np.where(np.arange(w) < w // 2, -0.5, 0.5)

    def with_split(D):
        h = hop_c.copy()
        h[i0] += np.diag(split * D)
        return h

    def gap_of(D):
        E = bands_on_mesh(with_split(D), rvec, rlat, kpt)
        return E[:, w // 2].min() - E[:, w // 2 - 1].max(), E

    lo, hi = 0.0, 1.0
    while gap_of(hi)[0] < gap:
        hi *= 2.0
    for _ in range(60):
        mid = 0.5 * (lo + hi)
        if gap_of(mid)[0] < gap:
            lo = mid
        else:
            hi = mid
    h = with_split(hi)
    g, E = gap_of(hi)
    efermi = 0.5 * (E[:, w // 2].min() + E[:, w // 2 - 1].max())
    spacing = float(np.min(np.diff(E, axis=1)))
    return h, float(efermi), spacing


def make_system(seed: int, w: int, lattice: str, rmax_steps: float, gap: float, ngrid,
                mshift=(0.0, 0.0, 0.0)) -> TBSystem:
    rng = np.random.default_rng(seed)
    if lattice == "hex":
        a = 3.2
        rlat = hex_lattice(a)
        rvec = lattice_vectors(rlat, rmax_steps * a, 2)
    elif lattice == "cubic":
        a = 5.0
        rlat = cubic_lattice(a)
        rvec = lattice_vectors(rlat, rmax_steps * a, 3)
    else:
        raise ValueError(lattice)
    Hc = random_hr(rng, w, rvec, rlat, a)
    kpt = monkhorst_pack(ngrid, rlat, mshift)
    Hc, efermi, _ = set_gap(Hc, rvec, rlat, kpt, gap)
    return TBSystem(w90basis=w, rvec=rvec, ffactor=np.ones(len(rvec), dtype=np.int32),
                    hop=np.ascontiguousarray(Hc.real), ihop=np.ascontiguousarray(Hc.imag),
                    rlat=rlat, efermi=efermi, scs=0.0, systype="2D" if lattice == "hex" else "3D")


def rk_params(ngrid, nc, nv, nev, r0=40.0) -> BSEParams:
    return BSEParams(ngrid=tuple(ngrid), nc=nc, nv=nv, coultype="V2DRK", ktol=1e-3,
                     ediel=(1.0, 1.0, 1.0), ez=1.0, w_coul=0.0, r0=r0, lc=1.0, cshift=0.05,
                     ebse0=0.0, ebsef=5.0, numbse=1000, nev=nev, renorm=True)


def workload(name: str, seed: int | None = None, params_only: bool = False):
    """The named workloads: returns (TBSystem, BSEParams); with params_only the system is not generated and
    (None, BSEParams) is returned.

    * ``hex8_24x24``   : 2D hexagonal, w=8, |R|<=3a (37), 24x24x1, 2v+2c, dim 2304, V2DRK r0=40 A,
                         10 excitons, spectrum 0-5 eV at 1000 points, CSHIFT 0.05.
    * ``cubic16_16x16x16``: simple cubic, w=16, |R|<=2a (33), 16^3, 3v+3c, dim 36,864, V3DL eps=8,
                         20 excitons.
    * ``hex12_60x60``  : 2D hexagonal, w=12, 60x60x1, 4v+4c, dim 57,600, V2DRK, 10 excitons.
    * ``hex8_36x36``   : 2D hexagonal, w=8, 36x36x1, 2v+2c, dim 5184, V2DRK, 4 excitons.
    * ``hex8_6x6``     : a small 2D case (dim 144) for fast checks.
    """
    if name == "hex8_24x24":
        spec, p = (11, 8, "hex", 3, 1.5, (24, 24, 1)), rk_params((24, 24, 1), 2, 2, 10)
    elif name == "cubic16_16x16x16":
        ng = (16, 16, 16)
        spec = (12, 16, "cubic", 2, 2.0, ng)
        p = BSEParams(ngrid=ng, nc=3, nv=3, coultype="V3DL", ktol=1e-3, ediel=(1.0, 8.0, 1.0),
                      cshift=0.05, ebse0=0.0, ebsef=5.0, numbse=1000, nev=20)
    elif name == "hex12_60x60":
        spec, p = (13, 12, "hex", 3, 1.5, (60, 60, 1)), rk_params((60, 60, 1), 4, 4, 10)
    elif name == "hex8_36x36":
        spec, p = (15, 8, "hex", 3, 1.5, (36, 36, 1)), rk_params((36, 36, 1), 2, 2, 4)
    elif name.startswith("hex"):
        # generic "hex{w}_{n}x{n}" with 2v+2c
        w_s, mesh = name[3:].split("_")
        n = int(mesh.split("x")[0])
        spec, p = (17, int(w_s), "hex", 3, 1.5, (n, n, 1)), rk_params((n, n, 1), 2, 2, 4)
    else:
        raise KeyError(name)
    if params_only:
        return None, p
    s0, w, lattice, rmax, gap, ng = spec
    return make_system(s0 if seed is None else seed, w, lattice, rmax, gap, ng), p


def system_from_arrays(a) -> TBSystem:
    """A TBSystem from stored arrays (a mapping such as an opened .npz with hop, ihop, rvec, ffactor, rlat,
    efermi and optionally scs and systype)."""
    keys = set(a.keys()) if hasattr(a, "keys") else set(a.files)
    return TBSystem(w90basis=int(a["hop"].shape[1]), rvec=np.ascontiguousarray(a["rvec"], dtype=np.int32),
                    ffactor=np.ascontiguousarray(a["ffactor"], dtype=np.int32),
                    hop=np.ascontiguousarray(a["hop"], dtype=np.float64),
                    ihop=np.ascontiguousarray(a["ihop"], dtype=np.float64),
                    rlat=np.ascontiguousarray(a["rlat"], dtype=np.float64), efermi=float(a["efermi"]),
                    scs=float(a["scs"]) if "scs" in keys else 0.0,
                    systype=str(a["systype"]) if "systype" in keys else "2D")


def strained_batch(seed: int = 14, nsys: int = 64, base_w: int = 8):
    """64 independent 2D systems: one seeded H(R) (w=8, gap 1.5 eV on a 24x24 mesh) plus per-system
    on-site strain shifts U(-0.2, 0.2) eV; meshes n x n with n in {12..36}; (nv, nc) in
    {(2,2), (3,3)}; 6 excitons each.  Returns a list of (TBSystem, BSEParams)."""
    base = make_system(seed, base_w, "hex", 3, 1.5, (24, 24, 1))
    rng = np.random.default_rng(seed + 1000)
    i0 = int(np.flatnonzero(np.all(base.rvec == 0, axis=1))[0])
    out = []
    for _ in range(nsys):
        s = base.copy()
        s.hop[i0] += np.diag(rng.uniform(-0.2, 0.2, base_w))
        n = int(rng.integers(12, 37))
        nb = 2 if rng.integers(0, 2) == 0 else 3
        ng = (n, n, 1)
        kpt = monkhorst_pack(ng, s.rlat)
        E = bands_on_mesh(s.hop + 1j * s.ihop, s.rvec, s.rlat, kpt)
        s.efermi = float(0.5 * (E[:, base_w // 2].min() + E[:, base_w // 2 - 1].max()))
        out.append((s, rk_params(ng, nb, nb, 6)))
    return out
