"""Build recipe for libpcgb300.so (sm_103a) -- nvcc only, no cmake.

Compiles the kernel translation units in parallel into ``_build/`` next to
this file and links them into ``_build/libpcgb300.so`` (plug-in entry points
with REAL = double) and ``_build/libpcgb300_sgl.so`` (the same library with
the runtime compiled for REAL = float, the single-precision Fortran build).
Re-running only recompiles sources newer than their objects.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpcgb300.so")
LIB_SGL = os.path.join(OUT, "libpcgb300_sgl.so")
# translation units compiled a second time for the single-precision plug-in
SGL_SOURCES = {"runtime.cu": "runtime_sgl.o"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["kernels_f32_7.cu", "kernels_f32_8.cu", "kernels_f64_7.cu", "kernels_f64_8.cu", "kernels_dd_7.cu",
           "kernels_dd_8.cu", "kernels_upw_f32.cu", "kernels_upw_f64.cu", "kernels_upw_dd_7.cu", "kernels_upw_dd_8.cu", "helical.cu", "cfl_pair.cu", "boundcond.cu",
           "aux_kernels.cu", "runtime.cu", "noalloc.cu", "server.cu"]
HEADERS = ["mhd_common.cuh", "mhd_driver.cuh", "cell_physics.cuh", "cell_scalar.cuh", "cell_pair.cuh", "kernels.cuh", "pcgb_box.h", "pcgb_ptx.cuh", "aux_kernels.h", "dd.cuh", "cell_ddpair.cuh", "helical.h", "cfl_pair.h", "boundcond.h", "params_check.h", "cell_pair_tmem.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpcgb300.so")


def _flags() -> list[str]:
    return ["-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
            "-I" + os.path.join(HERE, "..", "include")]


def _elf_machine_ok(path: str) -> bool:
    """True when an existing object/library was built for this machine's ISA."""
    want = {"x86_64": 62, "aarch64": 183, "arm64": 183}.get(os.uname().machine)
    try:
        with open(path, "rb") as fh:
            head = fh.read(20)
    except OSError:
        return False
    if len(head) < 20 or head[:4] != b"\x7fELF" or want is None:
        return False
    return int.from_bytes(head[18:20], "little") == want


def _newest_dep() -> float:
    deps = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "pcgb300.h")]
    return max(os.path.getmtime(d) for d in deps if os.path.exists(d))


def _compile(src: str, verbose: bool, obj_name: str | None = None, defines: tuple[str, ...] = ()) -> str:
    obj = os.path.join(OUT, obj_name or src.replace(".cu", ".o"))
    path = os.path.join(CSRC, src)
    if (os.path.exists(obj) and _elf_machine_ok(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(path), _newest_dep())):
        return obj
    cmd = [nvcc(), *_flags(), *[f"-D{d}" for d in defines], "-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def _link(lib: str, objs: list[str], verbose: bool) -> None:
    if (os.path.exists(lib) and _elf_machine_ok(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(o) for o in objs)):
        return
    cmd = [nvcc(), *ARCH, "-shared", "-o", lib, *objs, "-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")


def build(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    jobs = [(s, None, ()) for s in srcs] + [(s, o, ("PCGB_REAL_SINGLE",)) for s, o in SGL_SOURCES.items()]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(os.cpu_count() or 4, len(jobs)))) as ex:
        objs = list(ex.map(lambda j: _compile(j[0], verbose, j[1], j[2]), jobs))
    common = objs[:len(srcs)]
    sgl = objs[len(srcs):]
    _link(LIB, common, verbose)
    swap = {os.path.join(OUT, s.replace(".cu", ".o")): o for s, o in zip(SGL_SOURCES, sgl)}
    _link(LIB_SGL, [swap.get(o, o) for o in common], verbose)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
