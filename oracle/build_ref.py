"""Build recipe for the CPU oracle (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``oracle/espic_oracle.c`` into
  ``oracle/_build/libespic_oracle.so`` (runs everywhere, including the GPU
  host, because it needs nothing but gcc).
* ``build_reference()`` compiles the reference's own ch2, ch3/ver2 and ch4
  C++ sources, where they lie in the read-only reference checkout, together
  with the harnesses in ``oracle/ref_harness/`` into ``oracle/_ref/``.  It is
  skipped when the reference checkout is absent.  The reference is built as
  its README says (``g++ -O2``), plus ``-ffp-contract=off`` so that no
  multiply-add is fused on hosts whose base ISA has FMA.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: ESPIC_REFERENCE, else a sibling "reference" folder of
# the repository's parent (absent on hosts without it: build_reference skips)
REFERENCE = os.environ.get("ESPIC_REFERENCE",
                           os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference"))
ORACLE_SO = os.path.join(HERE, "_build", "libespic_oracle.so")

REF_TARGETS = {
    "ref_ch2": ("ch2", ["World.cpp", "Species.cpp", "PotentialSolver.cpp"], "ch2_harness.cpp"),
    "ref_ch3": ("ch3/ver2", ["World.cpp", "Species.cpp", "PotentialSolver.cpp", "Source.cpp"],
                "ch3_harness.cpp"),
    "ref_ch4": ("ch4", ["World.cpp", "Species.cpp", "Source.cpp", "Collisions.cpp"], "ch4_harness.cpp"),
    # the particle source of the MPI variant; its headers name MPI, which is
    # not installed, so a stand-in mpi.h (ref_harness/mpi_stub) satisfies them
    "ref_ch9mpi": ("ch9/MPI", ["src/Source.cpp", "src/World.cpp"], "ch9mpi_harness.cpp"),
}
EXTRA_INCLUDES = {"ref_ch9mpi": ["include", "@mpi_stub"]}


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_oracle(force=False):
    src = os.path.join(HERE, "espic_oracle.c")
    hdr = os.path.join(HERE, "espic_oracle.h")
    os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
    if force or _stale(ORACLE_SO, [src, hdr, __file__]):
        cmd = ["gcc", "-O2", "-std=c11", "-D_POSIX_C_SOURCE=200809L", "-ffp-contract=off", "-fPIC",
               "-shared", "-o", ORACLE_SO, src, "-lm", "-lpthread"]
        subprocess.check_call(cmd)
    return ORACLE_SO


def reference_available():
    return os.path.isdir(os.path.join(REFERENCE, "ch2"))


def ref_binary(name):
    return os.path.join(HERE, "_ref", name)


def build_reference(force=False):
    """Compile the reference harness binaries; returns {} if no reference."""
    if not reference_available():
        return {}
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    hdir = os.path.join(HERE, "ref_harness")
    built = {}
    procs = []
    for name, (chapter, files, harness) in REF_TARGETS.items():
        cdir = os.path.join(REFERENCE, chapter)
        srcs = [os.path.join(hdir, harness)] + [os.path.join(cdir, f) for f in files]
        out = os.path.join(outdir, name)
        built[name] = out
        deps = srcs + [os.path.join(hdir, "harness_io.h"), __file__]
        incs = ["-I", hdir, "-I", cdir]
        for d in EXTRA_INCLUDES.get(name, []):
            incs += ["-I", os.path.join(hdir, d[1:]) if d.startswith("@") else os.path.join(cdir, d)]
        if force or _stale(out, deps):
            cmd = ["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-w"] + incs + ["-o", out] + srcs
            procs.append((name, subprocess.Popen(cmd)))
    for name, p in procs:
        if p.wait() != 0:
            raise RuntimeError("reference harness %s failed to build" % name)
    return built


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
