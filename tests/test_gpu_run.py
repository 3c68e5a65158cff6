"""The run driver (pencil-code_gb300/run.py) on the reference samples' namelists:
time series every it1 steps, var.dat snapshots every dsnap, dim.dat, and the
same final state as stepping the box directly."""
import importlib
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _json(name):
    with open(os.path.join(GOLD, name)) as fh:
        return json.load(fh)


def test_run_driver_mhd_abcforcing(tmp_path, pc):
    run = importlib.import_module("pencil-code_gb300.run")
    vd = importlib.import_module("pencil-code_gb300.vardat")
    d = _json("mhd_abcforcing_ref.json")
    res = run.run(d["namelists"]["start.in"], d["namelists"]["run.in"], (32, 32, 32), str(tmp_path), nt=21)
    rows = res["rows"]
    assert [r["it"] for r in rows] == [0, 10, 20]
    assert rows[0]["t"] == 0.0 and rows[0]["urms"] == 0.0 and rows[0]["brms"] > 0.0
    assert all(r["dt"] > 0 for r in rows) and rows[1]["t"] > rows[0]["t"]
    lines = open(os.path.join(tmp_path, "data", "time_series.dat")).read().splitlines()
    assert lines[0].startswith("#") and len(lines) == 4
    mx, my, mz, mvar = vd.read_dim(os.path.join(tmp_path, "data", "dim.dat"))
    assert (mx, my, mz, mvar) == (38, 38, 38, 7)
    snap = vd.read_var(os.path.join(tmp_path, "data", "proc0", "var.dat"), mx, my, mz, mvar)
    # the same run stepped directly
    p = res["params"]
    q = pc.default_params()
    q.update(**p.as_dict())
    f0 = run.initial_state(q, {"initaa": "gaussian-noise", "amplaa": d["params"]["amplaa"]}, 1)
    box = pc.Box(q)
    box.load(f0)
    box.steps(21)
    assert np.array_equal(snap["f"], box.store())
    assert snap["t"] == box.time()[0]


def test_run_driver_helical_snapshots(tmp_path, pc):
    run = importlib.import_module("pencil-code_gb300.run")
    vd = importlib.import_module("pencil-code_gb300.vardat")
    d = _json("helical_mhdturb_ref.json")
    kd = d["kdat"]
    kdat = (np.array(kd["kxyz"]).reshape(3, kd["nk"]), kd["kav"])
    res = run.run(d["namelists"]["start.in"], d["namelists"]["run.in"], (32, 32, 32), str(tmp_path), kdat=kdat)
    ref = {r["it"]: r for r in d["series"]}
    rows = {r["it"]: r for r in res["rows"]}
    assert sorted(rows) == [0, 2, 4, 6, 8]
    # the state at t = 0.08 and 0.16 (rows it = 2, 4): one normalised forcing mode per step
    for it in (2, 4):
        assert abs(rows[it]["urms"] - ref[it]["urms"]) <= 5e-4 * ref[it]["urms"] + 1e-5, (it, rows[it])
    # dsnap = 0.1 over t = 0.4: a snapshot at the first step past each multiple of dsnap
    # (whether t = 0.4 itself counts depends on the last bit of t, as in the reference)
    names = sorted(os.path.basename(f) for f in res["files"])
    nsnap = len(names) - 2
    assert names[0] == "VAR0" and names[-1] == "var.dat" and nsnap in (3, 4)
    ts = [vd.read_var(os.path.join(tmp_path, "data", "proc0", f"VAR{i}"), 38, 38, 38, 7)["t"]
          for i in range(1, nsnap + 1)]
    assert all(abs(t - 0.04 * round(t / 0.04)) < 1e-12 for t in ts) and ts == sorted(ts)
    assert all(t >= 0.1 * (i + 1) - 1e-9 and t < 0.1 * (i + 1) + 0.04 + 1e-9 for i, t in enumerate(ts))


def test_run_driver_timing_namelists_with_boundaries(tmp_path, pc):
    """The timing run's namelists (upwinding, helical forcing of aa) with z made
    non-periodic ('s' for uu_x, uu_y, lnrho, A_x, A_y; 'a' for uu_z, A_z), on 24^3
    with a small forcing shell: VAR0 and var.dat carry the boundary ghosts, the grid
    record is the non-periodic one, and the final state is the box's own."""
    run = importlib.import_module("pencil-code_gb300.run")
    vd = importlib.import_module("pencil-code_gb300.vardat")
    nl = importlib.import_module("pencil-code_gb300.namelist")
    d = _json("timings_n4096_ref.json")
    start = d["namelists"]["start.in"].replace(
        "&init_pars", "&init_pars\n  lperi=T,T,F, bcz='s','s','a','s','s','s','a'", 1)
    kdat = nl.kvector_shell(8, 12)
    res = run.run(start, d["namelists"]["run.in"], (24, 24, 24), str(tmp_path), kdat=kdat, precision=4, nt=6)
    p = res["params"]
    assert p.lupw_uu == 1 and p.lmagnetic_forcing == 1 and not p.periodic(2)
    var = vd.read_var(os.path.join(tmp_path, "data", "proc0", "var.dat"), 30, 30, 30, 7)
    z = var["z"]
    assert abs(z[3] + np.pi) < 1e-12 and abs(z[26] - np.pi) < 1e-12   # points on both boundaries
    f = var["f"]
    # 's' mirrors, 'a' mirrors with a sign change about a zero boundary value; in the FP32
    # compensated state the interior is f + carry and a non-periodic ghost the condition
    # applied to f, so they agree to FP32 rounding
    def close(a, b):
        return np.max(np.abs(a - b)) <= 2e-7 * max(np.max(np.abs(b)), 1e-30)
    assert close(f[:, :, 2, 0], f[:, :, 4, 0]) and close(f[:, :, 27, 3], f[:, :, 25, 3])
    assert np.all(f[:, :, 3, 6] == 0.0) and close(f[:, :, 1, 6], -f[:, :, 5, 6])
    assert np.max(np.abs(f[3:-3, 3:-3, 3:-3, 4:7])) > 0.0   # aa forced
    v0 = vd.read_var(os.path.join(tmp_path, "data", "proc0", "VAR0"), 30, 30, 30, 7)
    assert np.all(np.isfinite(v0["f"])) and v0["t"] == 0.0
