"""var.dat snapshots and start.in/run.in namelists (host side, no GPU).

Pinned to fixtures made from the reference by tests/golden/gen_golden.py:
a var.dat committed with a reference sample run together with what the
reference's own record reader reads from it, and the MHD-ABCforcing sample's
namelist files.
"""
import hashlib
import importlib
import json
import os
import struct

import numpy as np
import pytest

vd = importlib.import_module("pencil-code_gb300.vardat")
nl = importlib.import_module("pencil-code_gb300.namelist")

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _json(name):
    with open(os.path.join(GOLD, name)) as fh:
        return json.load(fh)


def test_read_reference_sample_var():
    ref = _json("var_sample_1d.json")
    mx, my, mz, nv = ref["dim"]
    d = vd.read_var(os.path.join(GOLD, "var_sample_1d.dat"), mx, my, mz, nv, precision=8)
    assert d["f"].shape == (mx, my, mz, nv)
    assert d["t"] == ref["t"]
    assert d["x"].tolist() == ref["x"] and d["y"].tolist() == ref["y"] and d["z"].tolist() == ref["z"]
    assert [d["dx"], d["dy"], d["dz"]] == ref["dxyz"]
    assert d["f"][:, 1, 1, 0].tolist() == ref["f_row"]
    np.testing.assert_allclose(d["f"].sum(axis=(0, 1, 2)), ref["var_sums"], rtol=1e-14, atol=1e-12)
    assert np.abs(d["f"]).max(axis=(0, 1, 2)).tolist() == ref["var_absmax"]
    assert d["persistent"] == {}


def test_rewrite_reference_sample_is_byte_identical(tmp_path):
    ref = _json("var_sample_1d.json")
    mx, my, mz, nv = ref["dim"]
    src = os.path.join(GOLD, "var_sample_1d.dat")
    d = vd.read_var(src, mx, my, mz, nv)
    out = tmp_path / "var.dat"
    vd.write_var(str(out), d["f"], d["t"], d["x"], d["y"], d["z"], d["dx"], d["dy"], d["dz"])
    with open(src, "rb") as a, open(out, "rb") as b:
        assert a.read() == b.read()


def test_subrecords_match_reference_reader(tmp_path):
    ref = _json("var_subrecords.json")
    mx, my, mz, nv = ref["dim"]
    f = np.random.Generator(np.random.PCG64(ref["seed"])).standard_normal((mx, my, mz, nv))
    x, y, z = np.arange(mx) * 0.5, np.arange(my) * 0.25, np.arange(mz) * 0.125
    out = tmp_path / "var.dat"
    vd.write_var(str(out), f, 1.25, x, y, z, 0.5, 0.25, 0.125, max_subrecord=ref["max_subrecord"])
    assert os.path.getsize(out) == ref["file_bytes"]
    # markers: negative head while more subrecords follow, negative tail on continuations
    raw = out.read_bytes()
    heads, tails, o = [], [], 0
    while o < len(raw):
        h = struct.unpack("<i", raw[o:o + 4])[0]
        heads.append(h)
        tails.append(struct.unpack("<i", raw[o + 4 + abs(h):o + 8 + abs(h)])[0])
        o += 8 + abs(h)
    nsub = -(-f.nbytes // ref["max_subrecord"])
    assert all(h < 0 for h in heads[:nsub - 1]) and heads[nsub - 1] > 0
    assert tails[0] > 0 and all(t < 0 for t in tails[1:nsub])
    d = vd.read_var(str(out), mx, my, mz, nv)
    assert np.array_equal(d["f"], f)
    assert float(d["f"].sum()) == ref["ref_reader_sum"] and d["t"] == ref["ref_reader_t"]


def test_persistent_block_and_single_precision(tmp_path):
    f = np.arange(5 * 4 * 3 * 2, dtype=np.float32).reshape((5, 4, 3, 2), order="F")
    out = tmp_path / "var.dat"
    pers = {1: np.array([3.5], np.float32), 7: np.array([1, 2, 3], np.int32)}
    vd.write_var(str(out), f, 2.0, np.zeros(5), np.zeros(4), np.zeros(3), 1.0, 1.0, 1.0,
                 precision=4, persistent=pers)
    d = vd.read_var(str(out), 5, 4, 3, 2, precision=4)
    assert d["f"].dtype == np.float32 and np.array_equal(d["f"], f)
    assert set(d["persistent"]) == {1, 7}
    assert np.frombuffer(d["persistent"][7], np.int32).tolist() == [1, 2, 3]
    with pytest.raises(ValueError):
        vd.read_var(str(out), 5, 4, 3, 3, precision=4)


def test_corrupt_marker_is_an_error(tmp_path):
    out = tmp_path / "var.dat"
    vd.write_var(str(out), np.zeros((2, 2, 2, 1)), 0.0, np.zeros(2), np.zeros(2), np.zeros(2), 1, 1, 1)
    raw = bytearray(out.read_bytes())
    raw[4 + 64] ^= 0x01   # tail marker of the f record
    out.write_bytes(bytes(raw))
    with pytest.raises(ValueError):
        vd.read_var(str(out), 2, 2, 2, 1)


def test_box_snapshot_grid(tmp_path, pc):
    p = pc.default_params(nx=8, ny=6, nz=4)
    f = np.zeros(pc.host_shape(p), order="F")
    out = tmp_path / "var.dat"
    vd.write_box_snapshot(str(out), p, f, 0.5)
    d = vd.read_var(str(out), 14, 12, 10, 7)
    dx = 2 * np.pi / 8
    # cell centres of a periodic grid, ghosts included
    np.testing.assert_allclose(d["x"], -np.pi + (np.arange(14) - 2.5) * dx, rtol=0, atol=1e-15)
    assert d["dx"] == pytest.approx(dx, rel=1e-15) and d["t"] == 0.5


def test_namelists_of_mhd_abcforcing_sample():
    ref = _json("mhd_abcforcing_ref.json")
    par = ref["params"]
    p, ic, extra = nl.params_from_namelists(ref["namelists"]["start.in"], ref["namelists"]["run.in"],
                                            n=(par["n"],) * 3)
    assert (p.nx, p.ny, p.nz) == (32, 32, 32)
    assert p.gamma == par["gamma"] and p.nu == par["nu"] and p.eta == par["eta"]
    assert list(p.b_ext) == par["b_ext"] and p.cdt == par["cdt"]
    assert p.lforcing_cont == 1 and p.ampl_ff == par["ampl_ff"] and p.kf == par["k1_ff"]
    assert ic["initaa"] == par["initaa"] and ic["amplaa"] == par["amplaa"]
    assert ic["nt"] == par["nt"] and ic["it1"] == par["it1"]
    assert extra == {}


def test_namelist_lexical_rules():
    text = """
    ! comment line
    &run_pars
      dt=1.5d-3, nt=3*2   ! trailing comment
      name='a!b/c', flag=.false. , lst = 1, 2,
        3
    /
    &empty_pars /
    """
    g = nl.parse_namelists(text)
    assert g["run_pars"]["dt"] == 1.5e-3
    assert g["run_pars"]["nt"] == [2, 2, 2]
    assert g["run_pars"]["name"] == "a!b/c" and g["run_pars"]["flag"] is False
    assert g["run_pars"]["lst"] == [1, 2, 3]
    assert g["empty_pars"] == {}
    with pytest.raises(ValueError):
        nl.parse_namelists("&run_pars dt=1.0")


def test_namelist_unsupported_settings_are_errors():
    with pytest.raises(ValueError, match="itorder"):
        nl.params_from_namelists("", "&run_pars itorder=5 /")
    with pytest.raises(ValueError, match="bidiagonal"):
        nl.params_from_namelists("", "&run_pars lbidiagonal_derij=F /")
    with pytest.raises(ValueError, match="ABC"):
        nl.params_from_namelists("", "&hydro_run_pars lforcing_cont_uu=T / &forcing_run_pars lforcing_cont=T,"
                                     " iforcing_cont(1)='RobertsFlow' /")
    _, _, extra = nl.params_from_namelists("", "&viscosity_run_pars nu=0.01, nu_hyper3=1e-9 /")
    assert extra == {"viscosity_run_pars.nu_hyper3": 1e-9}


def test_namelists_of_helical_mhdturb_sample(tmp_path):
    ref = _json("helical_mhdturb_ref.json")
    p, ic, extra = nl.params_from_namelists(ref["namelists"]["start.in"], ref["namelists"]["run.in"], n=(32,) * 3)
    prm = ref["params"]
    assert p.lforcing_hel == 1 and p.force_hel == prm["force"] and p.relhel == prm["relhel"]
    assert p.nu == prm["nu"] and p.eta == prm["eta"] and p.dt == prm["dt"] and p.gamma == prm["gamma"]
    assert p.cdt == prm["cdt"] and p.cdtv == prm["cdtv"] and ic["nt"] == prm["nt"]
    assert "run_pars.random_gen" in extra
    # k.dat written back in the reference's format reads the same
    kd = ref["kdat"]
    kk = np.array(kd["kxyz"]).reshape(3, kd["nk"])
    path = tmp_path / "k.dat"
    with open(path, "w") as fh:
        fh.write(f"{kd['nk']} {kd['kav']}\n")
        for row in kk:
            fh.write(" ".join(str(int(v)) for v in row) + "\n")
    k2, kav = nl.read_kdat(str(path))
    assert kav == kd["kav"] and np.array_equal(k2, kk)
    with pytest.raises(ValueError, match="iforce"):
        nl.params_from_namelists("", "&forcing_run_pars iforce='irrotational' /")


def test_kvector_shells_match_reference_kdat():
    ref = _json("helical_mhdturb_ref.json")["kdat"]
    kv, kav = nl.kvector_shell(8, 12)
    assert kv.shape == (3, ref["nk"]) and np.array_equal(kv.ravel(), np.array(ref["kxyz"]))
    assert float("%.6g" % kav) == ref["kav"]
    t = _json("timings_n4096_ref.json")["kdat"]
    kv, kav = nl.kvector_shell(t["k2min"], t["k2max"])
    assert kv.shape == (3, t["nk"])
    digest = hashlib.sha256(kv.astype("<i2").tobytes()).hexdigest()
    assert digest == t["sha256_int16"]
    assert abs(kav - t["kav"]) < 1e-3


def test_namelists_of_timing_configuration():
    """doc/timings/N4096_32x32x32: upwinded advection and density, helical forcing of aa."""
    ref = _json("timings_n4096_ref.json")
    p, ic, extra = nl.params_from_namelists(ref["namelists"]["start.in"], ref["namelists"]["run.in"],
                                            n=(64, 64, 64), precision=4)
    assert p.lupw_uu == 1 and p.lupw_lnrho == 1
    assert p.lforcing_hel == 1 and p.lmagnetic_forcing == 1 and p.force_hel == 5e-4 and p.relhel == 1.0
    assert p.nu == 2e-5 and p.eta == 2e-5 and p.cdt == 0.9 and p.gamma == 1.0 and p.dt == 0.0
    assert ic["nt"] == 200 and ic["it1"] == 50 and ic["dsnap"] == 2.0
    # output-only switches are reported as not applied
    assert "magnetic_run_pars.lbb_as_aux" in extra and "run_pars.downsampl" in extra
    # its time series: the velocity is not forced, brms grows
    s = {r["it"]: r for r in ref["series"]}
    assert s[150]["urms"] == 0.0 and s[150]["brms"] > s[50]["brms"] > 0.0


def test_magnetic_forcing_options_are_checked():
    with pytest.raises(ValueError, match="lmagnetic_forcing"):
        nl.params_from_namelists("", "&forcing_run_pars lmagnetic_forcing=T /")
    with pytest.raises(ValueError, match="crosshel"):
        nl.params_from_namelists("", "&forcing_run_pars iforce='helical', lmagnetic_forcing=T, crosshel=1. /")
    with pytest.raises(ValueError, match="lhydro_forcing"):
        nl.params_from_namelists("", "&forcing_run_pars iforce='helical', lhydro_forcing=F /")
