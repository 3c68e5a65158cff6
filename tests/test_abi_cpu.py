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
    # the C ABI records a sticky error (the Python layer clears it once raised)
    assert not L.pcgb_box_create(C.byref(p))
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
    for bad in (dict(nx=2), dict(nx=5), dict(nz=4), dict(precision=2), dict(cdt=0.0), dict(cs0=-1.0),
                dict(dt=-1.0), dict(precision=4, dfloat=1), dict(dfloat=2)):
        p = pc.default_params(**bad)
        assert L.pcgb_set_params(C.byref(p)) != 0, bad


# Externals the reference's Fortran GPU module names (src/gpu_astaroth.f90:21-53),
# gfortran-mangled.  pos_real_ptr_c comes from src/syscalls_ansi.c:422, part of
# the reference's own syscalls object, not of the plug-in, and is left out.
FORTRAN_EXTERNALS = [
    "initialize_gpu_c", "register_gpu_c", "finalize_gpu_c", "get_farray_ptr_gpu_c", "rhs_gpu_c",
    "before_boundary_gpu_c", "update_after_substep_gpu_c", "radtransfer_gpu_c", "load_farray_c",
    "reload_gpu_config_c", "copy_farray_c", "update_on_gpu_arr_by_ind_c", "update_on_gpu_scal_by_ind_c",
    "update_on_gpu_vec_by_ind_c", "gpu_prepare_for_first_substep_c", "get_gpu_reduced_vars_c", "test_bcs_c",
    "split_update_gpu_c", "tf_train_c", "tf_infer_c", "tf_create_model_c", "print_snapshot_c",
    "tf_load_model_c", "tf_load_model_checkpoint_c", "tf_save_model_c", "tf_save_checkpoint_c",
    "update_on_gpu_arr_by_name_c", "update_on_gpu_scal_by_name_c", "update_on_gpu_vec_by_name_c",
]


def test_fortran_module_externals_link(pc):
    """A program naming every external of the Fortran GPU module links against the library alone."""
    lib_path = pc.load()._name
    decls = "\n".join(f"extern void {n}_(void);" for n in FORTRAN_EXTERNALS)
    refs = ", ".join(f"(void*){n}_" for n in FORTRAN_EXTERNALS)
    prog = f"{decls}\nvoid* table[] = {{{refs}}};\nint main(void) {{ return table[0] == 0; }}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "f.c")
        open(c, "w").write(prog)
        r = subprocess.run(["gcc", "-o", os.path.join(d, "f"), c, lib_path, "-Wl,--no-undefined"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_single_precision_plugin_library(pc):
    """libpcgb300_sgl.so, the plug-in for the reference's single-precision build
    (REAL = float): the same entry points as the double library, the Fortran
    externals link against it alone, and the header compiles with either REAL."""
    lib = importlib_lib(pc)
    S = lib.load_sgl()
    names = declared_functions()
    missing = [n for n in names if not hasattr(S, n)]
    assert not missing, missing
    assert S._name != pc.load()._name
    decls = "\n".join(f"extern void {n}_(void);" for n in FORTRAN_EXTERNALS)
    refs = ", ".join(f"(void*){n}_" for n in FORTRAN_EXTERNALS)
    prog = f"{decls}\nvoid* table[] = {{{refs}}};\nint main(void) {{ return table[0] == 0; }}\n"
    inc = os.path.join(os.path.dirname(__file__), "..", "include")
    hdr = ('#include "pcgb300.h"\n'
           '_Static_assert(sizeof(REAL_PCGB) == SZ, "REAL");\n'
           'void (*init)(REAL_PCGB*, int, double, int, int, int, int) = initializeGPU;\n'
           'void (*copy)(REAL_PCGB*) = copyFarray;\n'
           'int main(void) { return init == 0 || copy == 0; }\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "f.c")
        open(c, "w").write(prog)
        r = subprocess.run(["gcc", "-o", os.path.join(d, "f"), c, S._name, "-Wl,--no-undefined"],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        h = os.path.join(d, "h.c")
        open(h, "w").write(hdr)
        for define, size in (("", 8), ("-DPCGB_REAL_SINGLE", 4)):
            args = ["gcc", "-std=c11", "-I", inc, f"-DSZ={size}", "-o", os.path.join(d, "h"), h,
                    S._name if define else pc.load()._name, "-Wl,--no-undefined"]
            if define:
                args.insert(2, define)
            r = subprocess.run(args, capture_output=True, text=True)
            assert r.returncode == 0, (define, r.stderr)
