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
