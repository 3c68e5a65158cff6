"""Generate the golden vectors used by tests/test_oracle_golden.py.

Run where the pencil-code source tree is available (it is read here and
nowhere else), giving its path as the argument or in PENCIL_REFERENCE:

    python tests/golden/gen_golden.py <path of the pencil-code tree>

1. stencils.npz -- first and second derivatives of seeded random periodic
   fields computed by the reference's own numpy module
   python/pencil/math/derivatives/der_6th_order_w_ghosts.py (xder_6th ...
   zder2_6th), loaded standalone (the package-level import needs h5py).
2. mhd_abcforcing_ref.json -- the it / dt / urms / umax / brms columns of
   samples/MHD-ABCforcing/reference.out (and every column as printed text), the reference's regression series
   for isothermal MHD with continuous ABC forcing, with the run parameters of
   that sample's start.in / run.in, and the text of those two namelist files.
3. var_sample_1d.dat / var_sample_1d.json -- the var.dat snapshot committed
   with samples/1d-tests/axionSU2back_lhubble2 (data/proc0), copied as bytes,
   and what the reference's own Fortran record reader
   (python/pencil/read/fortran_file.py, FortranFileExt) reads from it.
5. helical_mhdturb_ref.json -- samples/helical-MHDturb: the wavevector list
   k.dat (random helical forcing), the it / t / dt / umax / urms columns of
   reference.out, the sample's run parameters and its start.in / run.in text.
4. var_subrecords.json -- a small snapshot written by
   pencil-code_gb300/vardat.py with a tiny subrecord size, checked at
   generation time to read back identically through FortranFileExt.
6. timings_n4096_ref.json -- doc/timings/N4096_32x32x32, the reference's
   timing configuration (upwinded advection, helical forcing of the vector
   potential): its start.in / run.in text, its time series, and its k.dat
   summarised as count, kav, the |k|^2 range and a SHA-256 of the vectors
   (int16, shape (3, nk)), so a regenerated shell can be checked against it.
"""
import hashlib
import importlib.util
import json
import os
import sys

import numpy as np

sys.dont_write_bytecode = True   # never write __pycache__ into the read-only tree


def load_der_module(ref_root):
    path = os.path.join(ref_root, "python", "pencil", "math", "derivatives", "der_6th_order_w_ghosts.py")
    spec = importlib.util.spec_from_file_location("ref_der6", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_fortran_file_module(ref_root):
    path = os.path.join(ref_root, "python", "pencil", "read", "fortran_file.py")
    spec = importlib.util.spec_from_file_location("ref_fortran_file", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def periodic(f):
    """Fill 3 ghost cells per side periodically; f indexed [z, y, x]."""
    for ax in range(3):
        n = f.shape[ax] - 6
        sl = [slice(None)] * 3
        src = [slice(None)] * 3
        sl[ax] = slice(0, 3); src[ax] = slice(n, n + 3)
        f[tuple(sl)] = f[tuple(src)]
        sl[ax] = slice(n + 3, n + 6); src[ax] = slice(3, 6)
        f[tuple(sl)] = f[tuple(src)]
    return f


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    m = load_der_module(ref_root)
    rng = np.random.Generator(np.random.PCG64(2024))
    nx, ny, nz = 12, 10, 8
    L = (2 * np.pi, 1.5 * np.pi, 2.5 * np.pi)
    dx, dy, dz = L[0] / nx, L[1] / ny, L[2] / nz
    out = {"n": np.array([nx, ny, nz]), "L": np.array(L)}
    for k in range(2):
        f = periodic(rng.standard_normal((nz + 6, ny + 6, nx + 6)))
        out[f"f{k}"] = f
        out[f"dx{k}"] = m.xder_6th(f, dx)[3:-3, 3:-3, 3:-3]
        out[f"dy{k}"] = m.yder_6th(f, dy)[3:-3, 3:-3, 3:-3]
        out[f"dz{k}"] = m.zder_6th(f, dz)[3:-3, 3:-3, 3:-3]
        out[f"dxx{k}"] = m.xder2_6th(f, dx)[3:-3, 3:-3, 3:-3]
        out[f"dyy{k}"] = m.yder2_6th(f, dy)[3:-3, 3:-3, 3:-3]
        out[f"dzz{k}"] = m.zder2_6th(f, dz)[3:-3, 3:-3, 3:-3]
    np.savez_compressed(os.path.join(here, "stencils.npz"), **out)

    # regression series of samples/MHD-ABCforcing (read as text)
    sample = os.path.join(ref_root, "samples", "MHD-ABCforcing")
    rows, printed = [], []
    with open(os.path.join(sample, "reference.out")) as fh:
        for line in fh:
            if line.startswith("#"):
                cols = [c for c in line.strip("#\n").split("-") if c]
                continue
            if not line.strip():
                continue
            v = line.split()
            rows.append({"it": int(v[0]), "t": float(v[1]), "dt": float(v[2]), "urms": float(v[3]),
                         "umax": float(v[4]), "brms": float(v[5])})
            # every column as printed, so a test can take its tolerance from the printed digits
            printed.append(dict(zip(cols, v)))
    params = {"n": 32, "gamma": 1.0, "nu": 0.1, "eta": 0.1, "ampl_ff": 1e-4, "k1_ff": 1.0,
              "iforcing_cont": "ABC", "b_ext": [0.0, 0.1, 0.0], "cdt": 0.4, "amplaa": 1e-2,
              "initaa": "gaussian-noise", "nt": 51, "it1": 10,
              "source": "samples/MHD-ABCforcing/{start.in,run.in,print.in,reference.out}"}
    namelists = {}
    for name in ("start.in", "run.in"):
        with open(os.path.join(sample, name)) as fh:
            namelists[name] = fh.read()
    with open(os.path.join(here, "mhd_abcforcing_ref.json"), "w") as fh:
        json.dump({"params": params, "series": rows, "printed": printed, "namelists": namelists}, fh, indent=1)

    # var.dat of a sample run, read by the reference's record reader
    ff = load_fortran_file_module(ref_root)
    sdir = os.path.join(ref_root, "samples", "1d-tests", "axionSU2back_lhubble2", "data")
    with open(os.path.join(sdir, "dim.dat")) as fh:
        mx, my, mz, mvar = (int(v) for v in fh.readline().split()[:4])
    src = os.path.join(sdir, "proc0", "var.dat")
    with open(src, "rb") as fh:
        raw = fh.read()
    with open(os.path.join(here, "var_sample_1d.dat"), "wb") as fh:
        fh.write(raw)
    fr = ff.FortranFileExt(src, header_dtype=np.int32)   # as varfile.py:838 opens it
    f = fr.read_record("<f8").reshape((mx, my, mz, mvar), order="F")
    g = fr.read_record("<f8")
    fr.close()
    summary = {"dim": [mx, my, mz, mvar], "precision": 8, "t": float(g[0]),
               "x": g[1:1 + mx].tolist(), "y": g[1 + mx:1 + mx + my].tolist(),
               "z": g[1 + mx + my:1 + mx + my + mz].tolist(),
               "dxyz": g[1 + mx + my + mz:4 + mx + my + mz].tolist(),
               "var_sums": f.sum(axis=(0, 1, 2)).tolist(), "var_absmax": np.abs(f).max(axis=(0, 1, 2)).tolist(),
               "f_row": f[:, 1, 1, 0].tolist(),
               "source": "samples/1d-tests/axionSU2back_lhubble2/data/{dim.dat,proc0/var.dat}"}
    with open(os.path.join(here, "var_sample_1d.json"), "w") as fh:
        json.dump(summary, fh, indent=1)

    # a snapshot written with forced subrecords, read back by the reference's reader
    sys.path.insert(0, os.path.dirname(os.path.dirname(here)))
    import importlib
    vd = importlib.import_module("pencil-code_gb300.vardat")
    mx, my, mz, nv = 9, 8, 7, 3
    rng = np.random.Generator(np.random.PCG64(7))
    f = rng.standard_normal((mx, my, mz, nv))
    x, y, z = np.arange(mx) * 0.5, np.arange(my) * 0.25, np.arange(mz) * 0.125
    tmp = os.path.join(here, "_subrec_tmp.dat")
    vd.write_var(tmp, f, 1.25, x, y, z, 0.5, 0.25, 0.125, max_subrecord=1000)
    fr = ff.FortranFileExt(tmp, header_dtype=np.int32)
    f2 = fr.read_record("<f8").reshape((mx, my, mz, nv), order="F")
    g2 = fr.read_record("<f8")
    fr.close()
    with open(tmp, "rb") as fh:
        size = len(fh.read())
    os.remove(tmp)
    assert np.array_equal(f2, f) and g2[0] == 1.25
    # helical forcing sample (k.dat and the regression series, read as text)
    hdir = os.path.join(ref_root, "samples", "helical-MHDturb")
    with open(os.path.join(hdir, "k.dat")) as fh:
        vals = fh.read().split()
    nk, kav = int(vals[0]), float(vals[1])
    kk = [float(v) for v in vals[2:2 + 3 * nk]]
    series = []
    with open(os.path.join(hdir, "reference.out")) as fh:
        for line in fh:
            if line.startswith("#") or not line.strip():
                continue
            v = line.split()
            series.append({"it": int(v[0]), "t": float(v[1]), "dt": float(v[2]), "umax": float(v[3]),
                           "urms": float(v[4])})
    hpar = {"n": 32, "gamma": 1.0, "nu": 5e-3, "eta": 5e-3, "iforce": "helical", "force": 0.07, "relhel": 1.0,
            "dt": 4e-2, "nt": 10, "it1": 2, "cdt": 0.4, "cdtv": 0.3,
            "source": "samples/helical-MHDturb/{start.in,run.in,k.dat,reference.out}"}
    hnl = {}
    for name in ("start.in", "run.in"):
        with open(os.path.join(hdir, name)) as fh:
            hnl[name] = fh.read()
    with open(os.path.join(here, "helical_mhdturb_ref.json"), "w") as fh:
        json.dump({"params": hpar, "kdat": {"nk": nk, "kav": kav, "kxyz": kk}, "series": series,
                   "namelists": hnl}, fh, indent=1)

    # the timing configuration of doc/timings (namelists, time series, k.dat digest)
    tdir = os.path.join(ref_root, "doc", "timings", "N4096_32x32x32")
    with open(os.path.join(tdir, "k.dat")) as fh:
        vals = fh.read().split()
    tnk, tkav = int(vals[0]), float(vals[1])
    tk = np.array([int(float(v)) for v in vals[2:2 + 3 * tnk]], dtype=np.int16).reshape(3, tnk)
    tk2 = (tk.astype(np.int64) ** 2).sum(0)
    tnl = {}
    for name in ("start.in", "run.in", "print.in"):
        with open(os.path.join(tdir, name)) as fh:
            tnl[name] = fh.read()
    tseries = []
    with open(os.path.join(tdir, "data", "time_series.dat")) as fh:
        cols = None
        for line in fh:
            if line.startswith("#"):
                cols = [c for c in line.strip("#\n").replace("-", " ").split()]
                continue
            v = line.split()
            tseries.append({c: (int(x) if c == "it" else float(x)) for c, x in zip(cols, v)})
    with open(os.path.join(tdir, "data", "dim.dat")) as fh:
        tdim = fh.read().split()
    with open(os.path.join(here, "timings_n4096_ref.json"), "w") as fh:
        json.dump({"kdat": {"nk": tnk, "kav": tkav, "k2min": int(tk2.min()), "k2max": int(tk2.max()),
                            "sha256_int16": hashlib.sha256(tk.astype("<i2").tobytes()).hexdigest()},
                   "namelists": tnl, "series": tseries,
                   "grid": {"nxgrid": 4096, "ncpus": 32768, "precision": tdim[6]},
                   "source": "doc/timings/N4096_32x32x32/{start.in,run.in,print.in,k.dat,data/time_series.dat,"
                             "data/dim.dat,src/cparam.local}"}, fh, indent=1)

    with open(os.path.join(here, "var_subrecords.json"), "w") as fh:
        json.dump({"dim": [mx, my, mz, nv], "seed": 7, "max_subrecord": 1000, "file_bytes": size,
                   "ref_reader_sum": float(f2.sum()), "ref_reader_t": float(g2[0])}, fh, indent=1)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PENCIL_REFERENCE")
    if not ref:
        sys.exit("usage: gen_golden.py <path of the pencil-code tree> (or set PENCIL_REFERENCE)")
    main(ref)
