"""Benchmark of the exciton path: BSE build + lowest-exciton solve on one GB300.

Metric: exciton solves/s (BSE build + lowest-10 solve) on the 2D hexagonal w=12, 60x60x1, 4v+4c system
(BSE dimension 57,600, Rytova-Keldysh r0 = 40 A), in the mixed-precision form (matrix-free operator,
split-BF16 tensor-core contraction, FP64 Rayleigh-Ritz and final refinement).  One step is one full
solve: H(k) and bands for the 3600 k-points, V(k,k') table, operator set-up, block eigensolve, oscillator
strengths.  The seeded system is the one stored with the FP64 oracle's results
(tests/golden/hex12_60x60_oracle.npz), so every exciton energy is reported with its error against the
oracle.  L2 is flushed (256 MB write) between timed steps.

Also reported in the same line:
  * the plain FP64 GPU forms of the same solve (dense FP64 build + FP64 operator; FP64 matrix-free operator),
    timed once each, with their errors against the oracle;
  * the end-to-end rate through the C ABI with host buffers (H(R) in, energies/activities/eigenvectors out);
  * the live-timed roofline of the dominant kernel (the tcgen05 contraction): algorithmic flops per launch
    (4 Nk^2 w^2 nb, one real-by-complex product) over the CUDA-event launch time against the measured burst
    bf16 peak; the issued split-BF16 work (three slice products) beside it;
  * the 3D cubic w=16 system (dim 36,864, lowest 20) in its FP64 GPU forms and the mixed form, and the
    64-system batch (systems/s);
  * a CPU baseline: the oracle's C restatement of the reference's path (element-by-element build, dense
    complex(8) matvecs, OpenMP on the host cores) timed on a bounded row sample and projected to one solve
    with the matvec count of a Krylov solve under the reference's SLEPc settings (oracle/krylov_counts.json).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--workload NAME]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "BSE build+solve s & exciton solves/s vs FP64 GPU path at 1e-5 eV error"
UNIT = "solves/s"
WORKLOADS = {
    "hex12_60x60": "2D hexagonal w=12, |R|<=3a (37 R), 60x60x1 k-mesh, 4v+4c, BSE dim 57600, V2DRK r0=40 A, "
                   "lowest 10 excitons",
    "hex8_24x24": "2D hexagonal w=8, |R|<=3a (37 R), 24x24x1 k-mesh, 2v+2c, BSE dim 2304, V2DRK r0=40 A, "
                  "lowest 10 excitons",
    "cubic16_16x16x16": "simple cubic w=16, |R|<=2a (33 R), 16^3 k-mesh, 3v+3c, BSE dim 36864, V3DL eps=8, "
                        "lowest 20 excitons",
    "batch64": "64 independent 2D hexagonal w=8 systems (on-site strain U(-0.2,0.2) eV), n x n meshes n in 12..36, "
               "(nv,nc) in {(2,2),(3,3)}, BSE dim 676..11664, lowest 6 excitons each",
}
GOLDEN = os.path.join(ROOT, "tests", "golden")


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region (into a temporary
    file that is removed afterwards)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="wtb_clocks_", suffix=".csv")
            self.f = os.fdopen(fd, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            lines = f.readlines()
        os.unlink(self.path)
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# the arithmetic of the exciton solve per precision form (operator / iteration, final Rayleigh-Ritz)
DTYPES = {"fp32": "f32 operator (FFT convolution on a 2D mesh), f32 iteration, f64 Rayleigh-Ritz",
          "bf16x3": "bf16x3+f32 operator, f64 Rayleigh-Ritz", "bf16x6": "bf16x6+f32 operator, f64 Rayleigh-Ritz",
          "fp64": "f64"}


def form_for(args, p, batch=False):
    """The precision form a workload runs in: the requested one, or with "auto" the fastest: fp32 where the FP32
    operator is the FFT convolution (a 2D mesh of at most 64 x 64 points), bf16x3 (tensor cores) otherwise and
    for the batch's joint graph."""
    if args.precision != "auto":
        return args.precision
    if batch:
        return "bf16x3"
    g = p.ngrid
    return "fp32" if (g[2] == 1 and max(g[0], g[1]) <= 64) else "bf16x3"


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


def load_workload(name):
    """(system, params, oracle fixture or None).  With a committed oracle fixture the system is the stored one
    (the generator's gap bisection calls LAPACK, whose last bits may differ between machines)."""
    from wtb_gb300 import synthetic as S

    path = os.path.join(GOLDEN, name + "_oracle.npz")
    if os.path.exists(path):
        g = np.load(path)
        _, p = S.workload(name, params_only=True)
        return S.system_from_arrays(g), p, g
    sysm, p = S.workload(name)
    return sysm, p, None


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_errors(ctx, p, out, g):
    """Per-eigenvalue |E - E_oracle| and the spectra's relative L2 error against the oracle fixture."""
    if g is None:
        return {}
    dE = np.abs(out["E"] - g["E"])
    spec = ctx.bsedielraw(p, out["Ws"], out["acts"])
    return {"dE_vs_oracle_eV": [float(x) for x in dE], "max_dE_vs_oracle_eV": float(dE.max()),
            "spectrum_rel_l2_vs_oracle": {c: rel_l2(spec[c][:, 2], g["spec_" + c][:, 2]) for c in ("xx", "yy", "zz")}}


# ----------------------------------------------------------------------------- CPU legs (oracle restatement)
def krylov_matvecs(name):
    """Matrix-vector products of one Krylov solve with the reference's SLEPc settings, measured on the oracle's
    operator by oracle/krylov_count.py (committed in oracle/krylov_counts.json)."""
    try:
        d = json.load(open(os.path.join(ROOT, "oracle", "krylov_counts.json")))[name]
        return int(d["matvecs"]), (f"{d['solver']}: nev={d['nev']}, ncv={d['ncv']}, tol={d['tol']}, "
                                   f"which={d['which']}, median of {len(d['runs'])} start vectors")
    except Exception:
        return None, None


class CpuReference:
    """The oracle's C restatement of the reference's path on the host cores: bands by LAPACK zheev per k-point,
    the element-by-element upper-triangle build (src/module_bse.F90:2399-2406) on a sample of rows, and a dense
    complex(8) matvec of that row block (the operation Krylov-Schur applies, src/module_slepc_solver.F90:44-74).
    A sample is projected to one solve: build x (elements of the upper triangle / elements built), matvec x
    (dim / rows) x the Krylov solve's matvec count."""

    MAX_BLOCK_BYTES = 4 << 30

    def __init__(self, sysm, p, matvecs):
        import ctypes

        import __graft_entry__ as g
        from oracle import wtb_oracle as O

        g.build_oracle()
        self.C = ctypes
        self.lib = ctypes.CDLL(g.ORACLE_SO)

        class Coul(ctypes.Structure):
            _fields_ = [("coultype", ctypes.c_int), ("ngrid", ctypes.c_int * 3), ("ktol", ctypes.c_double),
                        ("ediel", ctypes.c_double * 3), ("ez", ctypes.c_double), ("w", ctypes.c_double),
                        ("r0", ctypes.c_double), ("lc", ctypes.c_double), ("rlat", ctypes.c_double * 9)]

        cp = Coul()
        cp.coultype = {"V2DRK": 6, "V3DL": 2, "V3D": 1}[p.coultype]
        for i in range(3):
            cp.ngrid[i] = p.ngrid[i]
            cp.ediel[i] = p.ediel[i]
        cp.ktol, cp.ez, cp.w, cp.r0, cp.lc = p.ktol, p.ez, p.w_coul, p.r0, p.lc
        for i in range(9):
            cp.rlat[i] = float(sysm.rlat.reshape(-1)[i])
        self.cp = cp
        self.sysm, self.p, self.matvecs = sysm, p, matvecs
        self.dim = p.dim
        kpt = O.monhkhorst_pack(p.ngrid[0], p.ngrid[1], p.ngrid[2], p.mshift, sysm.rlat)
        t0 = time.perf_counter()
        eigv, vec, _ = O.bands(sysm, p, kpt)
        self.t_bands = time.perf_counter() - t0
        self.eigv, self.vec, self.kpt = (np.ascontiguousarray(a) for a in (eigv, vec, kpt))
        self.cores = int(self.lib.oracle_num_threads())
        self.rate = None  # seconds per built element
        self.block = None

    def _build(self, r0, rows):
        vp = self.C.c_void_p
        out = self.block[:rows]
        t0 = time.perf_counter()
        self.lib.oracle_build_rows(self.p.nk, self.p.nc, self.p.nv, self.sysm.w90basis, self.eigv.ctypes.data_as(vp),
                                   self.vec.ctypes.data_as(vp), self.kpt.ctypes.data_as(vp), self.C.byref(self.cp),
                                   self.C.c_long(r0), self.C.c_long(r0 + rows), out.ctypes.data_as(vp))
        return time.perf_counter() - t0

    def sample(self, budget_s, seed):
        """One bounded sample (about budget_s of CPU work): half building rows, half matvecs of the row block."""
        dim = self.dim
        max_rows = max(8, min(dim, self.MAX_BLOCK_BYTES // (16 * dim)))
        if self.block is None:
            self.block = np.zeros((max_rows, dim), dtype=np.complex128)
        rng = np.random.default_rng(seed)
        t_start = time.perf_counter()
        if self.rate is None:  # calibrate on a few rows
            n = min(8, dim)
            t = self._build(0, n)
            self.rate = t / sum(dim - i for i in range(n))
        rows = int(min(max_rows, max(8, (0.5 * budget_s / self.rate) / max(dim / 2, 1))))
        r0 = int(rng.integers(0, dim - rows + 1))
        tb = self._build(r0, rows)
        elems = rows * dim - (rows * (2 * r0 + rows - 1)) // 2  # sum over i in [r0, r0+rows) of dim - i
        self.rate = tb / elems
        vp = self.C.c_void_p
        x = np.ones((dim, 1), dtype=np.complex128)
        y = np.zeros((rows, 1), dtype=np.complex128)
        blk = self.block[:rows]
        t0 = time.perf_counter()
        reps = 0
        while reps < 1 or time.perf_counter() - t0 < 0.5 * budget_s:
            self.lib.oracle_dense_mv(self.C.c_long(rows), self.C.c_long(dim), blk.ctypes.data_as(vp),
                                     x.ctypes.data_as(vp), 1, y.ctypes.data_as(vp))
            reps += 1
        t_mv_rows = (time.perf_counter() - t0) / reps
        t_build = tb * (dim * (dim + 1) / 2.0) / elems
        t_mv = t_mv_rows * dim / rows
        t_solve = self.t_bands + t_build + self.matvecs * t_mv
        return {"t_sample_s": time.perf_counter() - t_start, "t_solve_s": t_solve, "t_build_s": t_build,
                "t_mv_s": t_mv, "rows": rows, "row0": r0, "elements": int(elems), "mv_reps": reps}

    def describe(self, s, source):
        return (f"oracle C restatement on {self.cores} threads: bands {self.t_bands:.2f} s (all {self.p.nk} "
                f"k-points, LAPACK zheev); element-by-element build of rows {s['row0']}..{s['row0'] + s['rows']} "
                f"of {self.dim} ({s['elements']} elements) projected to the upper triangle ({s['t_build_s']:.1f} s); "
                f"dense complex(8) matvec of that row block x{s['mv_reps']} projected to the full matrix "
                f"({s['t_mv_s']:.3f} s per matvec) x {self.matvecs} matvecs ({source}); "
                f"projected {s['t_solve_s']:.1f} s per solve")


def cpu_baseline(sysm, p, name, fallback_matvecs, budget_s):
    n, src = krylov_matvecs(name)
    if n is None:
        n, src = fallback_matvecs, "the FP64 GPU solve's operator applications (no committed Krylov count)"
    ref = CpuReference(sysm, p, n)
    ref.sample(0.25 * budget_s, seed=1)  # warm-up: page in the row block, settle the rate estimate
    s = ref.sample(budget_s, seed=0)
    return {"value": 1.0 / s["t_solve_s"], "unit": UNIT, "cores": ref.cores, "kind": "port", "projected": True,
            "sample": ref.describe(s, src), "sample_s": s["t_sample_s"], "projected_s_per_solve": s["t_solve_s"],
            "krylov_matvecs": n}


def run_reference(args):
    """The reference arm: the oracle's C restatement of the reference's CPU path (the reference itself needs
    Fortran, MPI, PETSc/SLEPc and MKL, none of which exists here or on the GPU machine), each step one bounded
    sample of the workload projected to one solve."""
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    name = args.workload if args.workload != "batch64" else "hex12_60x60"
    sysm, p, _ = load_workload(name)
    n, src = krylov_matvecs(name)
    if n is None:
        print(json.dumps({"impl": "reference", "unavailable": f"no committed Krylov matvec count for {name}"}))
        return 0
    ref = CpuReference(sysm, p, n)
    solves, sample_ms, last = [], [], None
    for i in range(args.warmup + args.steps):
        s = ref.sample(args.ref_budget, seed=1000 + i)
        if i >= args.warmup:
            solves.append(s["t_solve_s"])
            sample_ms.append(1000.0 * s["t_sample_s"])
        last = s
    v = float(args.steps / sum(solves))
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.mean(sample_ms)), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded H(R))",
            "impl": "reference", "projected": True,
            "step": "one bounded sample of the solve (rows of the element-by-element build and their dense "
                    "matvecs); ms_per_step is the sample's measured wall time, value the projected full solve",
            "projected_s_per_solve": float(np.mean(solves)),
            "config": {"workload": name, "description": WORKLOADS.get(name, name)},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": ref.cores, "kind": "port",
                             "sample": ref.describe(last, src)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------------------------- GPU legs
def batch_line(args, torch, api, S, world, local, steps, warmup):
    """systems/s over the 64-system batch: one step = the whole batch through wtb_batch_bsesolver (inputs
    staged from host memory, then one CUDA graph launch: per-system set-up branches, one joint eigensolve
    over all systems, per-system oscillator strengths; the call returns when every system is done)."""
    from wtb_gb300 import batch as B

    everything = S.strained_batch(nsys=64)
    rank = int(os.environ.get("RANK", "0"))
    # the 64 systems are split across ranks by the longest-processing-time partition (no collective on the
    # data path; only the step time is reduced)
    part = B.lpt_partition([B.system_cost(p, s.w90basis) for s, p in everything], world)[rank]
    items = [everything[i] for i in part]
    b = api.Batch(local)
    prec = form_for(args, None, batch=True)
    kw = dict(precision=prec, op="matfree", tol=args.tol)
    for _ in range(warmup):
        b.bsesolver(items, **kw)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = api.kernel_launch_count()
    side = torch.cuda.Stream()
    ms = []
    out = None
    for _ in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(side)
        out, _ = b.bsesolver(items, **kw)
        e1.record(side)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    launches = api.kernel_launch_count() - launches0
    clk = clocks.stop()
    tot = sum(ms)
    phases = b.timings()
    b.close()
    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([tot], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot = float(t.item())
    value = len(everything) * steps / (tot / 1000.0)
    h2d = sum(s.hop.nbytes + s.ihop.nbytes for s, _ in items)
    d2h = sum(p.nev * 8 * 9 for _, p in items)
    line = {"metric": "exciton systems/s (BSE build + lowest-6 solve, 64-system batch)", "value": value,
            "unit": "systems/s", "n_gpus": world, "steps": steps, "warmup": warmup,
            "ms_per_step": tot / steps, "higher_is_better": True, "scaling": "strong", "vs_baseline": None,
            "dtype": prec, "data": "synthetic (seeded H(R))",
            "config": {"workload": "batch64", "systems_this_rank": len(items), "sharding": "LPT over ranks",
                       "description": WORKLOADS["batch64"],
                       "form": "one graph launch per batch (joint ragged-batch eigensolve, grouped tcgen05 contraction)",
                       "precision": prec, "l2": "inputs and operators of 64 systems exceed L2 per step",
                       "timing": "events on a side stream around the blocking batch call"},
            "phases_ms": {k: round(v, 3) for k, v in phases.items()},
            "e2e": {"value": value, "unit": "systems/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches), "clocks": clk,
            "iterations": {"max": max(o["iterations"] for o in out), "mean": float(np.mean([o["iterations"] for o in out]))}}
    # the batch against its oracle fixture (a fixed subset of the systems, tests/golden/batch64_subset_oracle.npz)
    path = os.path.join(GOLDEN, "batch64_subset_oracle.npz")
    if os.path.exists(path) and world == 1:
        g = np.load(path)
        errs = {int(i): float(np.max(np.abs(out[int(i)]["E"] - g[f"E_{int(i)}"]))) for i in g["systems"]}
        line["max_dE_vs_oracle_eV"] = {"systems": errs, "max": max(errs.values())}
    return line


def timed_solves(torch, ctx, p, kw, steps, warmup, stream, l2buf, outs=None):
    for _ in range(warmup):
        ctx.bsesolver(p, **kw)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    last = None
    for i in range(steps):
        l2buf.fill_(1.0)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ev[i][0].record(stream)
        last = ctx.bsesolver(p, out=outs, **kw)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev], last


def once(torch, ctx, p, **kw):
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = ctx.bsesolver(p, **kw)
    torch.cuda.synchronize()
    return time.perf_counter() - t0, out


def fp64_forms(torch, ctx, p, g, t_mixed_s, last):
    """The plain FP64 GPU forms of the same solve, each timed once (wall, synchronised): the dense FP64 build +
    FP64 block matvecs, and the FP64 matrix-free operator (SIMT FP64 contraction).  Separates the precision
    gain from the matrix-free factorisation's."""
    res = {}
    for op in ("dense", "matfree"):
        t, out = once(torch, ctx, p, precision="fp64", op=op)
        d = {"build_plus_solve_s": t, "solves_per_s": 1.0 / t,
             "iterations": out["timings"]["iterations"], "matvec_columns": int(out["timings"]["matvec_columns"]),
             "max_abs_dE_eV_mixed_vs_this": float(np.max(np.abs(out["E"] - last["E"]))),
             "stage_ms": {k: out["timings"][k] for k in ("t_bands_ms", "t_build_ms", "t_solve_ms", "t_total_ms")}}
        if g is not None:
            d["max_dE_vs_oracle_eV"] = float(np.max(np.abs(out["E"] - g["E"])))
        res[op] = d
    return {"dense": res["dense"], "matfree": res["matfree"],
            "speedup_mixed_vs_fp64_dense": res["dense"]["build_plus_solve_s"] / t_mixed_s,
            "speedup_mixed_vs_fp64_matfree": res["matfree"]["build_plus_solve_s"] / t_mixed_s,
            "speedup_fp64_matfree_vs_fp64_dense": res["dense"]["build_plus_solve_s"] / res["matfree"]["build_plus_solve_s"]}


def contraction_roofline(api, ctx, p, kw, sysm, peaks, step_ms, last, precision):
    """The dominant kernel's live timing: one more (untimed) solve with the library's profile on; the eigensolve
    is a single graph launch, so the library times three launches of the iteration-phase contraction after it
    with CUDA events on its stream, the operator's data in place.  Called in isolation: the burst peak."""
    import ctypes

    api.lib().wtb_profile_enable(ctx._h, 1)
    ctx.bsesolver(p, **kw)
    tms, nl, fl, by = ctypes.c_double(), ctypes.c_longlong(), ctypes.c_double(), ctypes.c_double()
    api.lib().wtb_profile_read(ctx._h, ctypes.byref(tms), ctypes.byref(nl), ctypes.byref(fl), ctypes.byref(by))
    api.lib().wtb_profile_enable(ctx._h, 0)
    n = max(nl.value, 1)
    g_ms = tms.value / n
    issued = fl.value / n
    form = ctx.operator_form()
    if form == "FP32 FFT convolution":
        return fft_roofline(p, peaks, step_ms, last, g_ms, issued, by.value / n, int(nl.value))
    nk, w = p.nk, sysm.w90basis
    nb = 16  # the operator's block width (the eigensolver block)
    algo = 4.0 * nk * nk * w * w * nb  # one real V (nk x nk) times a complex panel (nk x w^2 nb)
    peak = peaks.get("bf16_tflops") if peaks else 1900.0
    ach = algo / (g_ms * 1e-3) / 1e12 if g_ms > 0 else None
    ach_issued = issued / (g_ms * 1e-3) / 1e12 if g_ms > 0 else None
    r = {"bound": "tensor", "kernel": "tc_gemm_kernel (tcgen05 split-BF16 V x Z contraction)",
         "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": (ach / peak) if ach else None,
         "peak_source": ("MEASURED_PEAKS.json bf16_tflops, the burst figure: the three launches are timed alone "
                         "(of measured)") if peaks else "fallback",
         "achieved_definition": "algorithmic flops 4*Nk^2*w^2*nb per launch (one real-by-complex product) / "
                                "CUDA-event launch time",
         "flops_algorithmic_per_launch": algo, "flops_issued_per_launch": issued,
         "issued_tflops": ach_issued, "frac_issued": (ach_issued / peak) if ach_issued else None,
         "issued_definition": "split-BF16: three bf16 slice products per real product",
         "launches_timed": int(nl.value), "avg_launch_ms": g_ms,
         "algorithmic_bytes_per_launch": by.value / n,
         "full_k_launches_per_step": last["timings"]["iterations"] + 2,
         "share_of_step": (g_ms * (last["timings"]["iterations"] + 2) / step_ms) if step_ms > 0 and g_ms > 0 else None,
         "traffic": None, "traffic_source": None}
    if precision not in ("bf16x3", "bf16x6"):
        r["bound"] = "simt"
    tr = os.path.join(ROOT, "profiles", "tc_gemm_traffic.json")
    if os.path.exists(tr):
        try:
            d = json.load(open(tr))
            r["traffic"] = d.get(p_name_of(p, sysm))
            r["traffic_source"] = d.get("source", "profiles/tc_gemm_traffic.json (an ncu capture, not this run)")
        except Exception:
            pass
    return r


# FP32 issue rate of the CUDA cores: 152 SMs x 128 lanes x 2 flops (FMA) at the 2070 MHz maximum SM clock
FP32_NOMINAL_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12


def fft_roofline(p, peaks, step_ms, last, g_ms, flops, algo_bytes, launches):
    """Roofline of the FP32 FFT convolution (the contraction of the FP32 matrix-free form on a 2D mesh): against
    the measured HBM copy rate with its algorithmic bytes (Z read and T written once in FP32, the P x P spectrum
    once), and its FFT flop rate (5 P log2 P per transform) against the CUDA cores' nominal FP32 rate."""
    hbm = peaks.get("hbm_gbs") if peaks else 6800.0
    ach = algo_bytes / (g_ms * 1e-3) / 1e9 if g_ms > 0 else None
    tfl = flops / (g_ms * 1e-3) / 1e12 if g_ms > 0 else None
    return {"bound": "hbm", "kernel": "fft_conv_kernel (FP32 FFT convolution of the gathered Z with the Coulomb "
                                      "stencil, one 128 x 128 transform pair per column pair)",
            "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": (ach / hbm) if ach else None,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback",
            "achieved_definition": "algorithmic bytes per launch (Z read and T written once in FP32, the spectrum "
                                   "once) / CUDA-event launch time",
            "algorithmic_bytes_per_launch": algo_bytes,
            "fft_flops_per_launch": flops, "fp32_tflops": tfl, "fp32_nominal_tflops": FP32_NOMINAL_TFLOPS,
            "frac_fp32_nominal": (tfl / FP32_NOMINAL_TFLOPS) if tfl else None,
            "limiter": "the shared-memory pipe (transposes and the transforms' passes through the shared grid), "
                       "not HBM: see profiles/fft_conv_hex12_60x60.md",
            "launches_timed": launches, "avg_launch_ms": g_ms,
            "launches_per_step": last["timings"]["iterations"] + 3,
            "share_of_step": (g_ms * (last["timings"]["iterations"] + 3) / step_ms) if step_ms > 0 and g_ms > 0
            else None,
            "traffic": FFT_TRAFFIC.get("hex12_60x60") if (p.nk == 3600 and p.ngrid[0] == 60) else None,
            "traffic_source": FFT_TRAFFIC.get("source") if p.nk == 3600 else "not captured for this workload"}


# DRAM bytes (read + write) of one fft_conv_kernel<128> launch on the 60 x 60 mesh from one ncu capture
# (profiles/fft_conv_hex12_60x60.md): below the algorithmic bytes because the L2 absorbs most of T's write
FFT_TRAFFIC = {"hex12_60x60": 66770176 + 19405568,
               "source": "profiles/fft_conv_hex12_60x60.md (an ncu --set full capture, not this run)"}


def p_name_of(p, sysm):
    return "hex12_60x60" if (p.nk == 3600 and sysm.w90basis == 12) else "other"


def c2_line(torch, api, ctx, args, stream, l2buf, local):
    """The 3D cubic w=16 system (dim 36,864, lowest 20, V3DL): its FP64 GPU forms and the mixed form, with
    per-eigenvalue errors against the oracle fixture."""
    name = "cubic16_16x16x16"
    sysm, p, g = load_workload(name)
    ctx.set_hr(sysm)
    prec = form_for(args, p)
    kw = dict(precision=prec, op="matfree", tol=args.tol)
    clocks = ClockSampler(local)
    clocks.start()
    ms, last = timed_solves(torch, ctx, p, kw, args.steps, args.warmup, stream, l2buf)
    clk = clocks.stop()
    step = float(np.mean(ms))
    d = {"workload": name, "description": WORKLOADS[name], "unit": UNIT, "value": 1000.0 / step,
         "ms_per_step": step, "steps": args.steps, "precision": prec, "contraction": ctx.operator_form(),
         "clocks": clk,
         "solver": {"iterations": last["timings"]["iterations"], "max_rel_residual": last["timings"]["max_rel_residual"]}}
    d.update(oracle_errors(ctx, p, last, g))
    d["fp64_gpu_form"] = fp64_forms(torch, ctx, p, g, step / 1000.0, last)
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300")
    ap.add_argument("--workload", default="hex12_60x60")
    ap.add_argument("--precision", default="auto",
                    help="auto (per workload: fp32 on a 2D mesh of at most 64 x 64 points, whose FP32 operator is the "
                         "FFT convolution, else bf16x3; bf16x3 for the batch), fp32, bf16x3, bf16x6 or fp64")
    ap.add_argument("--tol", type=float, default=0.0, help="residual target (0: the library's per-precision default)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 GPU forms")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-extra", action="store_true", help="skip the cubic and batch workloads")
    ap.add_argument("--ref-budget", type=float, default=4.0, help="seconds of CPU work per reference-arm sample")
    ap.add_argument("--cpu-budget", type=float, default=12.0, help="seconds of CPU work of the cpu_baseline sample")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from wtb_gb300 import api
    from wtb_gb300 import synthetic as S

    if args.workload == "batch64":
        line = batch_line(args, torch, api, S, world, local, args.steps, args.warmup)
        if rank == 0:
            print(json.dumps(line), flush=True)
        if world > 1:
            dist.destroy_process_group()
        return 0
    # one independent replica of the workload per GPU (systems are independent; no collective)
    sysm, p, g = load_workload(args.workload)
    ctx = api.Context(local)
    ctx.set_hr(sysm)
    stream = torch.cuda.ExternalStream(api.lib().wtb_ctx_stream(ctx._h))
    l2buf = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device=f"cuda:{local}")  # 256 MB > L2
    prec = form_for(args, p)
    solve_kw = dict(precision=prec, op="matfree", tol=args.tol)

    def pinned(shape, dtype, order="C"):
        n = int(np.prod(shape))
        t = torch.empty(n, dtype={np.float64: torch.float64, np.complex128: torch.complex128}[dtype], pin_memory=True)
        a = t.numpy()
        return a.reshape(shape[::-1]).T if order == "F" else a.reshape(shape)

    def pinned_copy(a):
        b = pinned(a.shape, np.float64, "F")
        b[...] = a
        return b

    # the solve's results (energies, activities and, end to end, the eigenvectors) land in page-locked memory
    outs = {"Ws": pinned((p.dim,), np.float64), "acts": pinned((p.dim, 8), np.float64, "F"),
            "HE": pinned((p.dim, p.nev), np.complex128, "F")}
    for _ in range(args.warmup):
        ctx.bsesolver(p, **solve_kw)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = api.kernel_launch_count()
    step_ms, last = timed_solves(torch, ctx, p, solve_kw, args.steps, 0, stream, l2buf, outs)
    launches = api.kernel_launch_count() - launches0
    clk = clocks.stop()
    tot_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([tot_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = float(t.item())
    value = world * args.steps / (tot_ms / 1000.0)
    mean_step = tot_ms / args.steps
    errs = oracle_errors(ctx, p, last, g)
    form = ctx.operator_form()
    roofline = contraction_roofline(api, ctx, p, solve_kw, sysm, measured_peaks(), mean_step, last, prec)

    # end to end through the C ABI with host buffers: H(R) host -> device, Ws/acts/HE device -> host, both in
    # page-locked host memory (allocated before the timed loop); every step of the device-timed loop again
    import dataclasses
    sys_pin = dataclasses.replace(sysm, hop=pinned_copy(np.asfortranarray(sysm.hop, dtype=np.float64)),
                                  ihop=pinned_copy(np.asfortranarray(sysm.ihop, dtype=np.float64)))
    e2e_ms = []
    for i in range(args.steps):
        l2buf.fill_(1.0)  # as between the device-timed steps; outside the timed window
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ctx.set_hr(sys_pin)
        ctx.bsesolver(p, want_vectors=True, out=outs, **solve_kw)
        torch.cuda.synchronize()
        e2e_ms.append(1000.0 * (time.perf_counter() - t0))
    h2d = sysm.hop.nbytes + sysm.ihop.nbytes + sysm.rvec.astype(np.int32).nbytes + \
        sysm.ffactor.astype(np.int32).nbytes + 9 * 8
    d2h = p.dim * 8 + p.dim * 8 * 8 + p.dim * p.nev * 16
    e2e = world * 1000.0 / float(np.mean(e2e_ms))

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mean_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": DTYPES.get(prec, prec),
            "data": "synthetic (seeded H(R), stored with the oracle's results)",
            "config": {"workload": args.workload, "description": WORKLOADS.get(args.workload, args.workload),
                       "operator": "matrix-free, contraction: " + form, "precision": prec,
                       "eigensolver_tol": args.tol,
                       "l2": "flushed between timed steps (256 MB write)", "parallelism": f"replicas x{world}"},
            "build_plus_solve_s": mean_step / 1000.0,
            **errs,
            "oracle": "tests/golden/%s_oracle.npz: ARPACK (tol 1e-10) on the FP64 factored operator" % args.workload
            if g is not None else None,
            "solver": {"iterations": last["timings"]["iterations"],
                       "matvec_columns": last["timings"]["matvec_columns"],
                       "max_rel_residual": last["timings"]["max_rel_residual"],
                       "fp64_refine_shift_eV": last["timings"]["refine_shift_max"],
                       "stage_ms": {k: last["timings"][k] for k in ("t_bands_ms", "t_build_ms", "t_solve_ms",
                                                                     "t_optics_ms", "t_total_ms")}},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "steps": len(e2e_ms)},
            "gpu_launches": int(launches), "roofline": roofline, "clocks": clk,
            "autotune": api.autotune_report()}

    fp64_cols = int(last["timings"]["matvec_columns"])
    if rank == 0 and not args.no_fp64:
        line["fp64_gpu_form"] = fp64_forms(torch, ctx, p, g, mean_step / 1000.0, last)
        fp64_cols = line["fp64_gpu_form"]["dense"]["matvec_columns"]
    if rank == 0 and not args.no_extra:
        line["workloads"] = {"cubic16_16x16x16": c2_line(torch, api, ctx, args, stream, l2buf, local)}
    ctx.close()
    if rank == 0 and not args.no_extra:
        line["workloads"]["batch64"] = batch_line(args, torch, api, S, 1, local, args.steps, args.warmup)
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(sysm, p, args.workload, fp64_cols, args.cpu_budget)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
