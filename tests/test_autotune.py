"""The autotuner of launch shapes (wtb_gb300/csrc/autotune.cu).

CPU: the report needs no device and names the source hash and the cache file the environment selects.
GPU (child processes, so that each starts with an empty in-process table): a first process measures the
matrix-free operator's contraction tile, gather tile and scatter column group and writes them to the JSON
cache; a second process reads them back and gets the same choices and bitwise the same energies; pinned
launch shapes at both ends of each candidate range give bitwise the same energies (no launch shape changes
the order of any sum).
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OPERATOR_PARAMS = ("tile_n", "gather_tile", "scatter_cols")


def test_report_needs_no_device(built):
    from wtb_gb300 import api

    r = api.autotune_report()
    assert set(r) == {"build", "cache", "choices"}
    assert len(r["build"]) == 16 and all(ch in "0123456789abcdef" for ch in r["build"])
    assert isinstance(r["choices"], list)


def test_cache_path_follows_the_environment(built, monkeypatch, tmp_path):
    from wtb_gb300 import api

    monkeypatch.setenv("WTB_TUNE_CACHE", "off")
    assert api.autotune_report()["cache"] is None
    monkeypatch.setenv("WTB_TUNE_CACHE", str(tmp_path / "t.json"))
    assert api.autotune_report()["cache"] == str(tmp_path / "t.json")
    monkeypatch.delenv("WTB_TUNE_CACHE")
    monkeypatch.setenv("XDG_CACHE_HOME", str(tmp_path / "xdg"))
    assert api.autotune_report()["cache"] == str(tmp_path / "xdg" / "wtb_gb300" / "autotune.json")
    monkeypatch.delenv("XDG_CACHE_HOME")
    monkeypatch.setenv("HOME", str(tmp_path / "home"))
    assert api.autotune_report()["cache"] == str(tmp_path / "home" / ".cache" / "wtb_gb300" / "autotune.json")


_CHILD = """
import json, sys
sys.path.insert(0, {root!r})
from wtb_gb300 import api, synthetic as S
sysm, p = S.workload("hex8_24x24")
ctx = api.Context(0)
ctx.set_hr(sysm)
r = ctx.bsesolver(p, precision="bf16x3", op="matfree")
print("RESULT " + json.dumps({{"E": [float(x) for x in r["E"]], "report": api.autotune_report()}}))
"""


def _solve_in_child(env_extra):
    env = dict(os.environ)
    env.pop("WTB_TC_TILE", None)
    env.pop("WTB_TUNE_PIN", None)
    env.pop("WTB_TUNE", None)
    env.update(env_extra)
    out = subprocess.run([sys.executable, "-c", _CHILD.format(root=ROOT)], env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stdout[-2000:] + out.stderr[-2000:]
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("RESULT ")][-1]
    d = json.loads(line[len("RESULT "):])
    choices = {c["param"]: c for c in d["report"]["choices"] if c["shape"].startswith("matfree ")}
    return np.array(d["E"]), choices, d["report"]


@pytest.mark.gpu
def test_choices_cached_and_reused(built, tmp_path):
    cache = tmp_path / "autotune.json"
    E1, ch1, rep1 = _solve_in_child({"WTB_TUNE_CACHE": str(cache)})
    for prm in OPERATOR_PARAMS:
        assert ch1[prm]["source"] == "measured", ch1
        assert len(ch1[prm]["ms"]) >= 2 and all(ms > 0 for _, ms in ch1[prm]["ms"])
        # the choice is the fastest measured candidate
        assert ch1[prm]["choice"] == min(ch1[prm]["ms"], key=lambda cm: cm[1])[0]
    doc = json.loads(cache.read_text())
    assert doc["format"] == "wtb_gb300 autotune 1"
    got = {e["param"]: e for e in doc["entries"] if e["shape"].startswith("matfree ")}
    for prm in OPERATOR_PARAMS:
        assert got[prm]["choice"] == ch1[prm]["choice"]
        assert got[prm]["build"] == rep1["build"] and "SMs" in got[prm]["device"]

    E2, ch2, _ = _solve_in_child({"WTB_TUNE_CACHE": str(cache)})
    for prm in OPERATOR_PARAMS:
        assert ch2[prm]["source"] == "cache"
        assert ch2[prm]["choice"] == ch1[prm]["choice"]
    np.testing.assert_array_equal(E2, E1)


@pytest.mark.gpu
def test_launch_shapes_leave_results_unchanged(built):
    pins = ("tile_n=128,gather_tile=801,scatter_cols=4", "tile_n=256,gather_tile=1604,scatter_cols=16")
    runs = [_solve_in_child({"WTB_TUNE_CACHE": "off", "WTB_TUNE_PIN": pin}) for pin in pins]
    for (E, ch, _), pin in zip(runs, pins):
        want = dict(kv.split("=") for kv in pin.split(","))
        for prm in OPERATOR_PARAMS:
            assert ch[prm]["source"] == "pinned" and ch[prm]["choice"] == int(want[prm]), (prm, ch)
    np.testing.assert_array_equal(runs[0][0], runs[1][0])


_CHILD_FFT = """
import json, sys
import numpy as np
sys.path.insert(0, {root!r})
from wtb_gb300 import api, synthetic as S
sysm, p = S.workload("hex8_24x24")
ctx = api.Context(0)
ctx.set_hr(sysm)
ctx.bsesolver(p, precision="fp64", op="matfree")
rng = np.random.default_rng(5)
X = rng.normal(size=(p.dim, 16)) + 1j * rng.normal(size=(p.dim, 16))
Y = ctx.bse_matvec(p, X, precision="fp32", op="matfree")
np.save({out!r}, Y)
print("RESULT " + json.dumps({{"form": ctx.operator_form(), "report": api.autotune_report()}}))
"""


@pytest.mark.gpu
def test_fft_launch_shapes_leave_results_unchanged(built, tmp_path):
    """The FFT form's gather and scatter: the row-per-thread tiles and the lane-k tiles (32 k along a warp's
    lanes) form every sum term for term in the same order, so H X is bitwise the same for every launch shape."""
    pins = ("gather_tile=1604,scatter_cols=2", "gather_tile=3201,scatter_cols=102",
            "gather_tile=3204,scatter_cols=108", "gather_tile=802,scatter_cols=104")
    Ys = []
    for i, pin in enumerate(pins):
        out = str(tmp_path / f"y{i}.npy")
        env = dict(os.environ)
        for k in ("WTB_TC_TILE", "WTB_TUNE_PIN", "WTB_TUNE", "WTB_FFT"):
            env.pop(k, None)
        env.update({"WTB_TUNE_CACHE": "off", "WTB_TUNE_PIN": pin})
        r = subprocess.run([sys.executable, "-c", _CHILD_FFT.format(root=ROOT, out=out)], env=env,
                           capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("RESULT ")][-1][len("RESULT "):])
        assert d["form"] == "FP32 FFT convolution"
        ch = {c["param"]: c for c in d["report"]["choices"] if c["shape"].startswith("matfree-fft ")}
        want = dict(kv.split("=") for kv in pin.split(","))
        for prm, v in want.items():
            assert ch[prm]["source"] == "pinned" and ch[prm]["choice"] == int(v), (prm, ch)
        Ys.append(np.load(out))
    for Y in Ys[1:]:
        np.testing.assert_array_equal(Y, Ys[0])
