"""In-tree build of libsm2d.so: the sm_103a CUDA kernels + C ABI; and of the
C++ drop-in layer over it (libsm2d_ref.so: the reference's pipeline and
wrapper entry points; libsm2d_ref_host.so: its grid and LUT types for programs
built without the reference's host code).

nvcc compiles the three CUDA translation units (the engine, the stage
entries and the redistribution surrogate) for sm_103a only, g++ compiles the host tables, the output writers
and the INI front end with -ffp-contract=off (so an Arm host gives the x86
float results), g++ links the shared library against the CUDA runtime, and
gcc builds the run_simulation command over it.  The compiles run in
parallel.  Usage: python -m sm_2d_gb300.build
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
SHIM = os.path.join(PKG, "shim")
OUT = os.path.join(PKG, "_lib")
LIB = os.path.join(OUT, "libsm2d.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home() -> str:
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _sources():
    return ([os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))] +
            [os.path.join(SHIM, f) for f in sorted(os.listdir(SHIM)) if f.endswith((".cpp", ".hpp"))] +
            [os.path.join(ROOT, "include", f) for f in ("sm2d.h", "sm2d_ref_types.hpp")])


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    inc = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
    cpp_units = ["sm2d_tables.cpp", "sm2d_output.cpp", "sm2d_config.cpp"]
    cpp_objs = [os.path.join(OUT, u.replace(".cpp", ".o")) for u in cpp_units]
    cu_units = ["sm2d_engine.cu", "sm2d_stages.cu", "sm2d_surrogate.cu"]
    cu_objs = [os.path.join(OUT, u.replace(".cu", ".o")) for u in cu_units]
    # --fmad=false: every float operation rounds on its own, as the oracle's
    # -ffp-contract=off build does, so that both transport passes (and the
    # oracle) take the same binning decisions from the same arithmetic
    cu_cmds = [[nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "--fmad=false", "-c", "-Xcompiler",
                "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr", *inc, os.path.join(CSRC, u), "-o", o]
               for u, o in zip(cu_units, cu_objs)]
    if ptxas_info:
        for c in cu_cmds:
            c.insert(1, "-Xptxas=-v")
    cpp_cmds = [["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", *inc, "-c", os.path.join(CSRC, u), "-o", o]
                for u, o in zip(cpp_units, cpp_objs)]

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or ptxas_info or r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError("build step failed: " + " ".join(cmd))
        return r

    with ThreadPoolExecutor(len(cu_cmds) + len(cpp_cmds)) as ex:
        for f in [ex.submit(run, c) for c in cu_cmds + cpp_cmds]:
            f.result()
    tmp = LIB + ".tmp"
    run(["g++", "-shared", "-o", tmp, *cu_objs, *cpp_objs, "-L" + os.path.join(cuda, "lib64"),
         "-L" + os.path.join(cuda, "targets", "sbsa-linux", "lib"), "-L" + os.path.join(cuda, "targets", "x86_64-linux", "lib"),
         "-lcudart", "-Wl,-rpath," + os.path.join(cuda, "lib64")])
    os.replace(tmp, LIB)
    # the run_simulation command over the library
    exe = os.path.join(OUT, "run_simulation")
    run(["gcc", "-O2", "-std=c11", *inc, os.path.join(CSRC, "sm2d_run_simulation.c"), "-o", exe + ".tmp",
         "-L" + OUT, "-lsm2d", "-Wl,-rpath,$ORIGIN"])
    os.replace(exe + ".tmp", exe)
    # the C++ drop-in layer: the reference's entry points over the C ABI
    cuda_inc = ["-I" + os.path.join(cuda, "include"), "-I" + os.path.join(cuda, "targets", "sbsa-linux", "include"),
                "-I" + os.path.join(cuda, "targets", "x86_64-linux", "include")]
    cuda_lib = ["-L" + os.path.join(cuda, "lib64"), "-L" + os.path.join(cuda, "targets", "sbsa-linux", "lib"),
                "-L" + os.path.join(cuda, "targets", "x86_64-linux", "lib")]
    for name, src, extra in (("libsm2d_ref.so", "sm2d_ref_shim.cpp", ["-lcudart"]),
                             ("libsm2d_ref_host.so", "sm2d_ref_grids.cpp", [])):
        out = os.path.join(OUT, name)
        run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", *inc, *cuda_inc, os.path.join(SHIM, src), "-o",
             out + ".tmp", "-L" + OUT, "-lsm2d", *cuda_lib, *extra, "-Wl,-rpath,$ORIGIN",
             "-Wl,-rpath," + os.path.join(cuda, "lib64")])
        os.replace(out + ".tmp", out)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True, ptxas_info="--ptxas" in sys.argv))
