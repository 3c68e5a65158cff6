"""The plug-in for the reference's single-precision build (libpcgb300_sgl.so,
REAL = float) against the double build's library.

Both run the same FP32 device state; the single-precision host array holds
float32(f0).  Loading converts float -> float in one library and
float64(float32) -> float in the other, so the device states agree bit for bit;
copyFarray rounds f + the compensation carry (summed in double) once to the
host REAL, so the float result is the double result rounded to float (1 ulp).
The reduced diagnostics are the double library's rounded to float.
"""
import ctypes as C
import importlib

import numpy as np
import pytest

from conftest import LOG7, oracle_params, rel_err

pytestmark = pytest.mark.gpu


def _run(L, real, f_host, p, nsteps, kvec=None):
    ptr = C.POINTER(real)
    assert L.pcgb_set_params(C.byref(p)) == 0
    if kvec is not None:
        kv = np.ascontiguousarray(kvec[0])
        assert L.pcgb_set_kvectors(kv.ctypes.data_as(C.POINTER(C.c_double)), kv.shape[1], kvec[1]) == 0
    L.initializeGPU(f_host.ctypes.data_as(ptr), 0, 0.0, 1, 0, 0, 0)
    assert L.pcgb_last_error() == 0
    for it in range(nsteps):
        if it == nsteps - 1:
            L.pcgb_request_diagnostics()
        for s in (1, 2, 3):
            L.substepGPU(s, 0.0)
    out = np.zeros_like(f_host, order="F")
    L.copyFarray(out.ctypes.data_as(ptr))
    red = np.zeros(20, dtype=f_host.dtype)
    L.getGPUReducedVars(red.ctypes.data_as(ptr))
    assert L.pcgb_last_error() == 0
    L.finalizeGPU()
    return out, red


@pytest.mark.parametrize("helical", [False, True])
def test_single_precision_plugin_matches_double_build(pc, ic, orc, helical):
    lib = importlib.import_module("pencil-code_gb300.lib")
    D, S = pc.load(), lib.load_sgl()
    p = pc.default_params(nx=40, ny=32, nz=24, gamma=1.0, nu=5e-3, eta=5e-3, dt=4e-3, precision=4, comp=1,
                          lforcing_cont=int(not helical), ampl_ff=0.02, kf=2.0)
    kvec = None
    if helical:
        nl = importlib.import_module("pencil-code_gb300.namelist")
        kvec = nl.kvector_shell(8, 12)
        p.update(lforcing_hel=1, force_hel=0.05, lmagnetic_forcing=1, lupw_uu=1, lupw_lnrho=1)
    f0 = ic.zeros(p)
    ic.gaussian_noise(f0, p, ["ux", "uy", "uz", "ax", "ay", "az"], 1e-2, 21)
    ic.fill_ghosts(f0)
    f32 = np.asfortranarray(f0.astype(np.float32))
    fd = np.asfortranarray(f32.astype(np.float64))
    out_d, red_d = _run(D, C.c_double, fd, p, 6, kvec)
    out_s, red_s = _run(S, C.c_float, f32, p, 6, kvec)
    assert out_s.dtype == np.float32
    # one rounding of the same double value
    assert np.array_equal(out_s, out_d.astype(np.float32))
    nz = red_d != 0
    assert np.array_equal(red_s[nz], red_d[nz].astype(np.float32))
    # and the single build's state against the FP64 oracle at the FP32 bar
    op = oracle_params(orc, p)
    f = np.array(fd, order="F", copy=True)
    df = np.zeros_like(f)
    t, dt, state = 0.0, p.dt, p.seed_ff
    for _ in range(6):
        if helical:
            rec, state = orc.helical_coefs(op, p.force_hel, kvec[0], kvec[1], state)
            _, state = orc.helical_coefs(op, p.force_hel, kvec[0], kvec[1], state)
        t, dt, _ = orc.time_step(op, f, df, t, dt, False, nthreads=8)
        if helical:
            orc.add_helical(op, f, rec, dt, 1)
            orc.ghosts(op, f)
    orc.ghosts(op, f)
    assert np.all(rel_err(out_s.astype(np.float64), f, LOG7) <= 1e-5)
