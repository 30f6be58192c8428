"""Build recipe for libespic.so (sm_103a only, no cmake).

Each .cu translation unit is compiled in parallel with nvcc for
arch=compute_103a, code=sm_103a, then linked into
plasma-simulations-by-example_gb300/_build/libespic.so.  k_fp64.cu is built with
-fmad=false so that its float64 arithmetic rounds every product and sum as the
reference's g++ build does; host code is built with -ffp-contract=off for the
same reason.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libespic.so")

UNITS = {
    "capi.cu": [],
    "k_fp64.cu": ["-fmad=false"],
    "k_mixed.cu": [],
    "k_pcg.cu": [],
    "noalloc.cu": ["-fmad=false"],
    "k_ensemble.cu": ["-fmad=false"],
    "adjoint.cu": [],
}


def nvcc():
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: libespic needs the CUDA toolkit")


def common_flags():
    return ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17",
            "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
            "-I", CSRC]


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    headers.append(os.path.join(ROOT, "include", "espic.h"))
    jobs = []
    objs = []
    for unit, flags in UNITS.items():
        src = os.path.join(CSRC, unit)
        obj = os.path.join(OUT, unit.replace(".cu", ".o"))
        objs.append(obj)
        if force or _stale(obj, [src, __file__] + headers):
            cmd = [cc, "-c", src, "-o", obj] + common_flags() + flags + list(extra)
            if verbose:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode:
                sys.stderr.write(r.stdout + r.stderr)
            if r.returncode:
                raise RuntimeError("nvcc failed: " + " ".join(cmd))
    if force or jobs or not os.path.exists(LIB):
        cmd = [cc, "-shared", "-o", LIB] + objs + ["-gencode", "arch=compute_103a,code=sm_103a",
                                                    "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError("link failed")
    return LIB


SHIM = os.path.join(PKG, "shim")
SHIM_LIB = os.path.join(OUT, "libespic_shim.a")


def build_shim(force=False):
    """The drop-in C++ classes (shim/espic_shim.cpp) as a static archive:
    link a reference Main.cpp with -lespic_shim -lespic."""
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(SHIM, "espic_shim.cpp")
    obj = os.path.join(OUT, "espic_shim.o")
    deps = [src, __file__, os.path.join(ROOT, "include", "espic.h")] + [
        os.path.join(SHIM, f) for f in os.listdir(SHIM) if f.endswith(".h")]
    if force or _stale(SHIM_LIB, deps):
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-c", src, "-o", obj, "-I", SHIM,
               "-I", os.path.join(ROOT, "include")]
        subprocess.check_call(cmd)
        if os.path.exists(SHIM_LIB):
            os.remove(SHIM_LIB)
        subprocess.check_call(["ar", "rcs", SHIM_LIB, obj])
    return SHIM_LIB


def compile_drop_in(main_source, out, stdin_source=False):
    """Compile a program written against the reference's headers (World.h,
    Species.h, ...) with the drop-in headers and link libespic.  With
    stdin_source the file is fed on stdin from an empty directory, so that
    its own directory's headers are not found first."""
    build(False)
    build_shim(False)
    cmd = ["g++", "-O2", "-std=c++17", "-x", "c++", "-I", SHIM, "-I", os.path.join(ROOT, "include")]
    cmd += ["-"] if stdin_source else [main_source]
    cmd += ["-x", "none", SHIM_LIB, "-L", OUT, "-lespic", "-Wl,-rpath," + OUT, "-o", out]
    if stdin_source:
        import tempfile
        with tempfile.TemporaryDirectory() as td, open(main_source) as f:
            return subprocess.run(cmd, stdin=f, cwd=td, capture_output=True, text=True)
    return subprocess.run(cmd, capture_output=True, text=True)


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
    print(build_shim(force="--force" in sys.argv))
