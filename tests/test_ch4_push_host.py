"""The GPU path's per-particle ch4 neutral push (csrc/ch4_push.h), compiled
as host code with nvcc, against the oracle's restatement (pinned bit for bit
to the reference by test_oracle_golden.py::test_ch4_neutral_push_bitexact):
five steps of tests/golden/ch4_push.npz (3000 atoms, ~120 sphere bounces)
with the reference's uniforms.  Removing the dead in the CUDA path's order
(the oracle's holes mode), positions, velocities and the survivor order
agree bit for bit (host math library on both sides)."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden

PD = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    out = str(tmp_path_factory.mktemp("ch4host") / "libch4host.so")
    csrc = os.path.join(ROOT, "plasma-simulations-by-example_gb300", "csrc")
    subprocess.run([nvcc, "-shared", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-O2", "-I", csrc,
                    "-gencode", "arch=compute_103a,code=sm_103a", "-o", out,
                    os.path.join(ROOT, "tests", "ch4_push_host.cu")], check=True, capture_output=True)
    L = C.CDLL(out)
    L.ch4_host_step.restype = C.c_int64
    L.ch4_host_step.argtypes = [PD, PD, PD, C.c_double, C.c_double, PD, C.c_int64, C.c_int64, PD, PD,
                                C.POINTER(C.c_int64), C.POINTER(C.c_int32)]
    return L


def pd(a):
    return a.ctypes.data_as(PD)


def test_ch4_push_core_matches_oracle(host_lib, po):
    f = golden("ch4_push")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    sph = f["sphere"]
    s4 = np.array([sph[0], sph[1], sph[2], sph[3] ** 2])
    x0, xm = np.array(f["x0"], dtype=float), np.array(f["xm"], dtype=float)
    mass, dt = float(f["mass"]), float(f["dt"])
    P, pdt, off, bounces = f["P0"].copy(), f["dt0"].copy(), 0, 0
    for _ in range(int(f["steps"])):
        u = np.ascontiguousarray(f["u"][off:])
        want, want_pdt, used, p_off = po.advance_ch4_neutral(g, tuple(sph[:4]), mass, dt, P, pdt, u, holes=True)
        Q = np.ascontiguousarray(P.copy())
        alive = np.zeros(Q.shape[1], dtype=np.int32)
        b = host_lib.ch4_host_step(pd(x0), pd(xm), pd(s4), mass, dt, pd(Q), Q.shape[1], Q.shape[1], pd(pdt), pd(u),
                                   p_off.ctypes.data_as(C.POINTER(C.c_int64)),
                                   alive.ctypes.data_as(C.POINTER(C.c_int32)))
        assert 11 * b == used
        # the CUDA path's removal order
        n_alive = int(alive.sum())
        Q[6] = np.where(alive == 1, Q[6], 0.0)
        hole = 0
        for src in range(n_alive, Q.shape[1]):
            if not alive[src]:
                continue
            while alive[hole]:
                hole += 1
            Q[:, hole] = Q[:, src]
            alive[hole] = 1
            hole += 1
        got = Q[:, :n_alive]
        assert got.shape == want.shape and np.array_equal(got, want)
        off += used
        bounces += b
        P, pdt = want, want_pdt
    assert bounces > 50
