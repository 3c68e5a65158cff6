"""The C-ABI library on a machine without a GPU: it loads, exports every entry
point include/pcgb300.h declares, its parameter block has the same layout in
C and in the ctypes mirror, and calls that need a GPU fail with an error code
instead of computing anything on the CPU."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pcgb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M):
        name = m.group(1)
        if name not in ("if", "while", "return", "sizeof"):
            names.add(name)
    return sorted(names)


def test_library_exports_every_declared_symbol(pc):
    L = pc.load()
    names = declared_functions()
    assert len(names) > 80
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    lib = importlib_lib(pc)
    assert set(lib.EXPORTS) <= set(names)


def importlib_lib(pc):
    import importlib
    return importlib.import_module("pencil-code_gb300.lib")


def test_params_layout_matches_c(pc):
    lib = importlib_lib(pc)
    fields = [f for f, _ in lib.Params._fields_]
    prog = ["#include <stdio.h>", "#include <stddef.h>", f'#include "{HEADER}"', "int main(void){",
            'printf("%zu\\n", sizeof(pcgb_params));']
    for f in fields:
        prog.append(f'printf("%zu\\n", offsetof(pcgb_params, {f}));')
    prog.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        open(c, "w").write("\n".join(prog))
        exe = os.path.join(d, "l")
        subprocess.run(["gcc", "-o", exe, c], check=True)
        out = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    assert out[0] == C.sizeof(lib.Params)
    for f, off in zip(fields, out[1:]):
        assert getattr(lib.Params, f).offset == off, f


def test_default_params_are_reference_defaults(pc):
    p = pc.default_params()
    assert (p.cdt, p.cdtv) == (0.9, 0.25)                   # cdata.f90:235,239
    assert abs(p.gamma - 5.0 / 3.0) < 1e-15                  # eos_idealgas.f90:47
    assert list(p.xyz0) == [-np.pi] * 3 and list(p.Lxyz) == [2 * np.pi] * 3   # cdata.f90:211
    assert (p.relhel, p.abc_a, p.abc_b, p.abc_c, p.ampl_fcont_uu) == (1.0, 1.0, 1.0, 1.0, 1.0)
    assert (p.lohmic_heat, p.lviscosity_heat) == (1, 1)      # magnetic.f90:247, entropy.f90:139


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="checks the no-GPU failure path")
def test_no_cpu_fallback_without_gpu(pc):
    L = pc.load()
    p = pc.default_params(nx=16, ny=16, nz=16, dt=1e-3)
    with pytest.raises(pc.PcgbError):
        pc.Box(p)
    rc = L.pcgb_last_error()
    assert rc != 0 and L.pcgb_error_string(rc)
    # the plug-in path records an error and computes nothing
    assert L.pcgb_set_params(C.byref(p)) == 0
    f = np.zeros((22, 22, 22, 7), order="F")
    L.pcgb_clear_error()
    L.initializeGPU(f.ctypes.data_as(C.POINTER(C.c_double)), 0, 0.0, 1, 0, 0, 0)
    assert L.pcgb_last_error() != 0
    L.pcgb_clear_error()
    L.substepGPU(1, 0.0)
    assert L.pcgb_last_error() != 0


def test_parameter_validation(pc):
    L = pc.load()
    for bad in (dict(nx=2), dict(precision=2), dict(cdt=0.0), dict(cs0=-1.0), dict(dt=-1.0)):
        p = pc.default_params(**bad)
        assert L.pcgb_set_params(C.byref(p)) != 0, bad
