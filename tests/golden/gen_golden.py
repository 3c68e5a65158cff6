"""Generate the golden vectors used by tests/test_oracle_golden.py.

Run in a container where the reference tree is mounted (it is read here and
nowhere else):

    python tests/golden/gen_golden.py /root/reference

1. stencils.npz -- first and second derivatives of seeded random periodic
   fields computed by the reference's own numpy module
   python/pencil/math/derivatives/der_6th_order_w_ghosts.py (xder_6th ...
   zder2_6th), loaded standalone (the package-level import needs h5py).
2. mhd_abcforcing_ref.json -- the it / dt / urms / umax / brms columns of
   samples/MHD-ABCforcing/reference.out, the reference's regression series
   for isothermal MHD with continuous ABC forcing, with the run parameters of
   that sample's start.in / run.in.
"""
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
    rows = []
    with open(os.path.join(sample, "reference.out")) as fh:
        for line in fh:
            if line.startswith("#") or not line.strip():
                continue
            v = line.split()
            rows.append({"it": int(v[0]), "t": float(v[1]), "dt": float(v[2]), "urms": float(v[3]),
                         "umax": float(v[4]), "brms": float(v[5])})
    params = {"n": 32, "gamma": 1.0, "nu": 0.1, "eta": 0.1, "ampl_ff": 1e-4, "k1_ff": 1.0,
              "iforcing_cont": "ABC", "b_ext": [0.0, 0.1, 0.0], "cdt": 0.4, "amplaa": 1e-2,
              "initaa": "gaussian-noise", "nt": 51, "it1": 10,
              "source": "samples/MHD-ABCforcing/{start.in,run.in,print.in,reference.out}"}
    with open(os.path.join(here, "mhd_abcforcing_ref.json"), "w") as fh:
        json.dump({"params": params, "series": rows}, fh, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
