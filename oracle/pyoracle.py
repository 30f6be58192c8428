"""ctypes view of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loaded by the tests, the smoke check and the CPU-baseline leg of bench.py,
as the checker; the product library never imports it.  Arrays follow the
oracle's conventions: node fields in U order (i fastest), ef as [nn, 3],
particles as a (7, n) float64 block x, y, z, vx, vy, vz, mpw.
"""
import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np

from . import build_ref

_lib = None

D = C.c_double
I64 = C.c_int64
PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)
PI64 = C.POINTER(C.c_int64)


class Grid(C.Structure):
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("pad", C.c_int),
                ("x0", D * 3), ("xm", D * 3), ("dh", D * 3)]

    @property
    def nn(self):
        return self.ni * self.nj * self.nk


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build_oracle()
        _lib = C.CDLL(path)
        _sig(_lib)
    return _lib


def _sig(L):
    L.eo_philox_uniform.restype = D
    L.eo_philox_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
    L.eo_philox_uniforms.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, I64, PD]
    L.eo_grid_set.argtypes = [C.POINTER(Grid), C.c_int, C.c_int, C.c_int, PD, PD]
    L.eo_node_volumes.argtypes = [C.POINTER(Grid), PD]
    L.eo_push_box.argtypes = [C.POINTER(Grid), PD, D, D, D, PD, I64, I64]
    L.eo_push_sphere.restype = I64
    L.eo_push_sphere.argtypes = [C.POINTER(Grid), PD, PD, D, D, D, PD, I64, I64]
    L.eo_compact_swap_last.restype = I64
    L.eo_compact_swap_last.argtypes = [PD, I64, I64]
    L.eo_compact_holes.restype = I64
    L.eo_compact_holes.argtypes = [PD, I64, I64]
    L.eo_add_particles.restype = I64
    L.eo_add_particles.argtypes = [C.POINTER(Grid), PD, D, D, D, PD, PD, PD, I64, PD, I64, I64, I64]
    L.eo_load_box.restype = I64
    L.eo_load_box.argtypes = [C.POINTER(Grid), PD, D, D, D, PD, PD, D, I64, PD, PD, I64, I64, I64]
    L.eo_load_box_qs.restype = I64
    L.eo_load_box_qs.argtypes = [C.POINTER(Grid), PD, D, D, D, PD, PD, D, PI, PD, I64, I64, I64]
    L.eo_load_box_thermal.restype = I64
    L.eo_load_box_thermal.argtypes = [C.POINTER(Grid), PD, D, D, D, PD, PD, D, I64, PD, D, PD, PD, I64, I64,
                                      I64]
    L.eo_inject_count.restype = C.c_int
    L.eo_inject_count.argtypes = [C.POINTER(Grid), D, D, D, D, D]
    L.eo_inject_cold.restype = I64
    L.eo_inject_cold.argtypes = [C.POINTER(Grid), PD, D, D, D, D, D, D, PD, PI64, PD, I64, I64, I64]
    L.eo_inject_beam.restype = I64
    L.eo_inject_beam.argtypes = [C.POINTER(Grid), PD, D, D, D, D, D, D, D, C.c_int, PD, PD, PI64, PD, I64, I64,
                                 I64]
    L.eo_dsmc_mex.restype = I64
    L.eo_dsmc_mex.argtypes = [C.POINTER(Grid), D, D, D, PD, PD, PD, I64, I64, PD, I64, PI64, PI64]
    L.eo_sample_moments.argtypes = [C.POINTER(Grid), PD, I64, I64, PD]
    L.eo_gas_properties.argtypes = [C.POINTER(Grid), D, PD, PD, PD]
    L.eo_compute_mpc.argtypes = [C.POINTER(Grid), PD, I64, I64, PD]
    L.eo_mcc_cex.restype = I64
    L.eo_mcc_cex.argtypes = [C.POINTER(Grid), PD, I64, I64, PD, PD, D, PD, I64, PI64, PI64]
    L.eo_chemistry_ionize.restype = I64
    L.eo_chemistry_ionize.argtypes = [C.POINTER(Grid), PD, PD, PD, D, D, D, D, D, PD, I64, PD, PD, I64, PI64]
    L.eo_advance_ch4_ion.restype = I64
    L.eo_advance_ch4_ion.argtypes = [C.POINTER(Grid), PD, PD, D, D, D, D, PD, I64, I64, PD, D, D, D, D, D, D, PD,
                                     I64, C.POINTER(C.c_int32), PD, PI64, PD, I64, PI64]
    L.eo_advance_ch4_neutral.restype = I64
    L.eo_advance_ch4_neutral.argtypes = [C.POINTER(Grid), PD, D, D, PD, I64, I64, PD, PD, I64, PI64, PI64, C.c_int]
    L.eo_inject_warm.restype = I64
    L.eo_inject_warm.argtypes = [C.POINTER(Grid), PD, D, D, D, D, D, D, D, PD, PI64, PD, I64, I64,
                                 I64]
    L.eo_deposit_fp64.argtypes = [C.POINTER(Grid), PD, I64, I64, PD]
    L.eo_deposit_fixed.argtypes = [C.POINTER(Grid), PD, I64, I64, D, PI64]
    L.eo_divide_volume.argtypes = [I64, PD, PD]
    L.eo_density_from_fixed.argtypes = [I64, PI64, D, PD, PD]
    L.eo_charge_density.argtypes = [I64, C.c_int, PD, PD, PD]
    L.eo_fixed_scale_exponent.restype = C.c_int
    L.eo_fixed_scale_exponent.argtypes = [D, I64]
    L.eo_residual_box.restype = D
    L.eo_residual_box.argtypes = [C.POINTER(Grid), PD, PD]
    for f in (L.eo_sor_box_lex, L.eo_sor_box_rb):
        f.restype = C.c_int
        f.argtypes = [C.POINTER(Grid), PD, PD, C.c_int, D, PD, PI]
    L.eo_objects_sphere.argtypes = [C.POINTER(Grid), PD, D, D, PI, PD]
    L.eo_objects_inlet.argtypes = [C.POINTER(Grid), PI, PD]
    L.eo_neumann_targets.argtypes = [C.POINTER(Grid), PI, PI]
    L.eo_residual_sphere.restype = D
    L.eo_residual_sphere.argtypes = [C.POINTER(Grid), PD, PD, PI, D, D, D]
    L.eo_gs_sphere_lex.restype = C.c_int
    L.eo_gs_sphere_lex.argtypes = [C.POINTER(Grid), PD, PD, PI, D, D, D, C.c_int, D, PD, PI]
    L.eo_sor_sphere_rb.restype = C.c_int
    L.eo_sor_sphere_rb.argtypes = [C.POINTER(Grid), PD, PD, PI, PI, D, D, D, C.c_int, D, PD, PI]
    L.eo_qn.argtypes = [C.POINTER(Grid), PD, PD, PI, D, D, D]
    L.eo_newton_pcg.restype = C.c_int
    L.eo_newton_pcg.argtypes = [C.POINTER(Grid), PD, PD, PI, PI, D, D, D, C.c_int, D, C.c_int, D,
                                PI, PI]
    L.eo_efield.argtypes = [C.POINTER(Grid), PD, PD]
    L.eo_species_diag.argtypes = [PD, I64, I64, D, PD]
    L.eo_potential_energy.restype = D
    L.eo_potential_energy.argtypes = [C.POINTER(Grid), PD, PD]
    L.eo_update_average.argtypes = [I64, PD, PD, C.c_int]
    L.eo_bench_push_deposit.restype = D
    L.eo_bench_push_deposit.argtypes = [C.POINTER(Grid), PD, PD, D, D, D, D, PD, I64, I64, C.c_int,
                                        C.c_int, PI64, PI64]


def pd(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(PD)


def pi(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(PI)


def pi64(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(PI64)


def arr3(v):
    return (D * 3)(*[float(x) for x in v])


def grid(n, x0, xm):
    g = Grid()
    lib().eo_grid_set(C.byref(g), int(n[0]), int(n[1]), int(n[2]), arr3(x0), arr3(xm))
    return g


def node_volumes(g):
    v = np.zeros(g.nn)
    lib().eo_node_volumes(C.byref(g), pd(v))
    return v


def philox_uniforms(seed, stream, first, n):
    out = np.zeros(int(n))
    lib().eo_philox_uniforms(seed, stream, first, int(n), pd(out))
    return out


def push_box(g, ef, charge, mass, dt, P):
    P = np.ascontiguousarray(P, dtype=np.float64).copy()
    lib().eo_push_box(C.byref(g), pd(ef), charge, mass, dt, pd(P), P.shape[1], P.shape[1])
    return P


def push_sphere(g, ef, sphere4, charge, mass, dt, P, compact="swap_last"):
    P = np.ascontiguousarray(P, dtype=np.float64).copy()
    n = P.shape[1]
    s = np.asarray(sphere4, dtype=np.float64)
    L = lib()
    L.eo_push_sphere(C.byref(g), pd(ef), pd(s), charge, mass, dt, pd(P), n, n)
    if compact == "swap_last":
        m = L.eo_compact_swap_last(pd(P), n, n)
    elif compact == "holes":
        m = L.eo_compact_holes(pd(P), n, n)
    else:
        return P
    return np.ascontiguousarray(P[:, :m])


def add_particles(g, ef, charge, mass, dt, pos3, vel3, w, P=None, cap=None):
    pos3 = np.ascontiguousarray(pos3, dtype=np.float64)
    vel3 = np.ascontiguousarray(vel3, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    n = pos3.shape[0]
    np0 = 0 if P is None else P.shape[1]
    cap = cap or (np0 + n)
    B = np.zeros((7, cap))
    if P is not None:
        B[:, :np0] = P
    m = lib().eo_add_particles(C.byref(g), pd(ef), charge, mass, dt, pd(pos3), pd(vel3), pd(w), n,
                               pd(B), cap, np0, cap)
    return np.ascontiguousarray(B[:, :m])


def load_box(g, ef, charge, mass, dt, x1, x2, num_den, num_mp, u):
    B = np.zeros((7, num_mp))
    u = np.ascontiguousarray(u, dtype=np.float64)
    m = lib().eo_load_box(C.byref(g), pd(ef), charge, mass, dt, arr3(x1), arr3(x2), num_den, num_mp,
                          pd(u), pd(B), num_mp, 0, num_mp)
    return np.ascontiguousarray(B[:, :m])


def load_box_qs(g, ef, charge, mass, dt, x1, x2, num_den, num_mp):
    cap = int(np.prod(num_mp))
    B = np.zeros((7, cap))
    nm = np.asarray(num_mp, dtype=np.int32)
    m = lib().eo_load_box_qs(C.byref(g), pd(ef), charge, mass, dt, arr3(x1), arr3(x2), num_den,
                             pi(nm), pd(B), cap, 0, cap)
    return np.ascontiguousarray(B[:, :m])


def load_box_thermal(g, ef, charge, mass, dt, x1, x2, mpw, num_mp, vd, temp, u):
    B = np.zeros((7, num_mp))
    u = np.ascontiguousarray(u, dtype=np.float64)
    m = lib().eo_load_box_thermal(C.byref(g), pd(ef), charge, mass, dt, arr3(x1), arr3(x2), mpw, num_mp,
                                  arr3(vd), temp, pd(u), pd(B), num_mp, 0, num_mp)
    return np.ascontiguousarray(B[:, :m])


def inject(g, ef, charge, mass, dt, mpw0, v_drift, den, u, temp=None, P=None):
    u = np.ascontiguousarray(u, dtype=np.float64)
    L = lib()
    cnt = L.eo_inject_count(C.byref(g), dt, mpw0, v_drift, den, float(u[0]))
    np0 = 0 if P is None else P.shape[1]
    cap = np0 + max(cnt, 0)
    B = np.zeros((7, max(cap, 1)))
    if P is not None:
        B[:, :np0] = P
    used = C.c_int64(0)
    if temp is None:
        m = L.eo_inject_cold(C.byref(g), pd(ef), charge, mass, dt, mpw0, v_drift, den, pd(u),
                             C.byref(used), pd(B), B.shape[1], np0, B.shape[1])
    else:
        m = L.eo_inject_warm(C.byref(g), pd(ef), charge, mass, dt, mpw0, v_drift, den, temp, pd(u),
                             C.byref(used), pd(B), B.shape[1], np0, B.shape[1])
    return np.ascontiguousarray(B[:, :m]), used.value


def inject_beam(g, ef, charge, mass, dt, mpw0, v_drift, den, temp, mode, u, rem=None, max_new=100000):
    """eo_inject_beam: mode 2 (ch9/MPI isotropic) or 3 (Maxwellian); with rem
    (a one-element float64 array) the remainder count, updated in place."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    B = np.zeros((7, max_new))
    used = C.c_int64(0)
    rp = None if rem is None else rem.ctypes.data_as(PD)
    m = lib().eo_inject_beam(C.byref(g), pd(ef), charge, mass, dt, mpw0, v_drift, den, temp, mode, rp, pd(u),
                             C.byref(used), pd(B), B.shape[1], 0, B.shape[1])
    assert m >= 0
    return np.ascontiguousarray(B[:, :m]), used.value


def dsmc_mex(g, mass, mpw0, dt, c, sigma_cr_max, P, u):
    """eo_dsmc_mex: one DSMC_MEX::apply on a copy of P with the uniforms u.
    Returns (P after, sigma_cr_max after, collisions, uniforms used, the
    per-cell offsets of the first uniform, n_cells + 1 entries)."""
    P = np.array(P, dtype=np.float64, order="C", copy=True)
    u = np.ascontiguousarray(u, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    smax = np.array([sigma_cr_max], dtype=np.float64)
    ncell = (g.ni - 1) * (g.nj - 1) * (g.nk - 1)
    off = np.zeros(ncell + 1, dtype=np.int64)
    used = C.c_int64(0)
    ncol = lib().eo_dsmc_mex(C.byref(g), mass, mpw0, dt, pd(c), pd(smax), pd(P), P.shape[1], P.shape[1], pd(u),
                             u.size, C.byref(used), off.ctypes.data_as(PI64))
    assert ncol >= 0, "uniforms ran out"
    return P, float(smax[0]), int(ncol), used.value, off


def sample_moments(g, P, mom=None):
    """eo_sample_moments: adds P's samples to mom (7 planes of nn: n, nu, nv,
    nw, nuu, nvv, nww; zeros when None) and returns it."""
    P = np.ascontiguousarray(P, dtype=np.float64)
    nn = g.ni * g.nj * g.nk
    mom = np.zeros(7 * nn) if mom is None else np.ascontiguousarray(mom, dtype=np.float64).copy()
    lib().eo_sample_moments(C.byref(g), pd(P), P.shape[1], P.shape[1], pd(mom))
    return mom


def gas_properties(g, mass, mom):
    """eo_gas_properties: (vel [nn][3] flattened, T [nn])"""
    nn = g.ni * g.nj * g.nk
    mom = np.ascontiguousarray(mom, dtype=np.float64)
    vel, T = np.zeros(3 * nn), np.zeros(nn)
    lib().eo_gas_properties(C.byref(g), mass, pd(mom), pd(vel), pd(T))
    return vel, T


def compute_mpc(g, P):
    P = np.ascontiguousarray(P, dtype=np.float64)
    mpc = np.zeros((g.ni - 1) * (g.nj - 1) * (g.nk - 1))
    lib().eo_compute_mpc(C.byref(g), pd(P), P.shape[1], P.shape[1], pd(mpc))
    return mpc


def mcc_cex(g, P, den, vel, dt, u):
    """eo_mcc_cex on a copy of P: (P after, collisions, uniforms used, the
    per-particle offset of its uniform in u)"""
    P = np.array(P, dtype=np.float64, order="C", copy=True)
    u = np.ascontiguousarray(u, dtype=np.float64)
    den = np.ascontiguousarray(den, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    off = np.zeros(max(P.shape[1], 1), dtype=np.int64)
    used = C.c_int64(0)
    ncol = lib().eo_mcc_cex(C.byref(g), pd(P), P.shape[1], P.shape[1], pd(den), pd(vel), dt, pd(u), u.size,
                            C.byref(used), off.ctypes.data_as(PI64))
    return P, int(ncol), used.value, off[:P.shape[1]]


def advance_ch4_neutral(g, sphere, mass, dt, P, pdt, u, holes=False):
    """eo_advance_ch4_neutral on copies of P and pdt: (P, pdt after removal,
    uniforms used, each particle's first uniform index).  sphere: (cx, cy,
    cz, radius).  holes=True removes the dead in the CUDA path's order."""
    P = np.array(P, dtype=np.float64, order="C", copy=True)
    pdt = np.array(pdt, dtype=np.float64, copy=True)
    u = np.ascontiguousarray(u, dtype=np.float64)
    sph = np.array(list(sphere[:3]) + [sphere[3] ** 2], dtype=np.float64)
    used = C.c_int64(0)
    off = np.zeros(max(P.shape[1], 1), dtype=np.int64)
    m = lib().eo_advance_ch4_neutral(C.byref(g), pd(sph), mass, dt, pd(P), P.shape[1], P.shape[1], pd(pdt), pd(u),
                                     u.size, C.byref(used), off.ctypes.data_as(PI64), 1 if holes else 0)
    assert m >= 0, "uniforms ran out"
    return np.ascontiguousarray(P[:, :m]), pdt[:m].copy(), used.value, off[:P.shape[1]]


def chemistry_ionize(g, den_n, rho, ef, charge, mass, mpw0, rate, dt, u, max_new=200000):
    """eo_chemistry_ionize: (new ions [7][m], their time left, uniforms used)"""
    den_n, rho, ef = (np.ascontiguousarray(a, dtype=np.float64) for a in (den_n, rho, ef))
    u = np.ascontiguousarray(u, dtype=np.float64)
    Q, qdt = np.zeros((7, max_new)), np.zeros(max_new)
    used = C.c_int64(0)
    m = lib().eo_chemistry_ionize(C.byref(g), pd(den_n), pd(rho), pd(ef), charge, mass, mpw0, rate, dt, pd(Q),
                                  max_new, pd(qdt), pd(u), u.size, C.byref(used))
    assert m >= 0, "uniforms ran out or the buffer of new particles is full"
    return np.ascontiguousarray(Q[:, :m]), qdt[:m].copy(), used.value


def advance_ch4_ion(g, ef, sphere, charge, mass, mpw0, dt, P, pdt, neutral, spherium, u, max_new=100000):
    """eo_advance_ch4_ion on copies of P and pdt.  neutral, spherium:
    (mpw0, charge, mass) of the target species.  Returns (P, pdt after
    removal, created particles [7][m], their tags (0 neutral, 1 spherium),
    their time left, uniforms used)."""
    P = np.array(P, dtype=np.float64, order="C", copy=True)
    pdt = np.array(pdt, dtype=np.float64, copy=True)
    u = np.ascontiguousarray(u, dtype=np.float64)
    ef = np.ascontiguousarray(ef, dtype=np.float64)
    sph = np.array(list(sphere[:3]) + [sphere[3] ** 2], dtype=np.float64)
    Q = np.zeros((7, max_new))
    tag = np.zeros(max_new, dtype=np.int32)
    qdt = np.zeros(max_new)
    m, used = C.c_int64(0), C.c_int64(0)
    npart = lib().eo_advance_ch4_ion(C.byref(g), pd(ef), pd(sph), charge, mass, mpw0, dt, pd(P), P.shape[1],
                                     P.shape[1], pd(pdt), neutral[0], neutral[1], neutral[2], spherium[0],
                                     spherium[1], spherium[2], pd(Q), max_new,
                                     tag.ctypes.data_as(C.POINTER(C.c_int32)), pd(qdt), C.byref(m), pd(u), u.size,
                                     C.byref(used))
    assert npart >= 0, "uniforms ran out or the buffer of new particles is full"
    k = m.value
    return (np.ascontiguousarray(P[:, :npart]), pdt[:npart].copy(), np.ascontiguousarray(Q[:, :k]), tag[:k].copy(),
            qdt[:k].copy(), used.value)


def deposit_fp64(g, P):
    P = np.ascontiguousarray(P, dtype=np.float64)
    acc = np.zeros(g.nn)
    lib().eo_deposit_fp64(C.byref(g), pd(P), P.shape[1], P.shape[1], pd(acc))
    return acc


def deposit_fixed(g, P, fx):
    P = np.ascontiguousarray(P, dtype=np.float64)
    acc = np.zeros(g.nn, dtype=np.int64)
    lib().eo_deposit_fixed(C.byref(g), pd(P), P.shape[1], P.shape[1], fx, pi64(acc))
    return acc


def divide_volume(den, vol):
    den = np.ascontiguousarray(den, dtype=np.float64).copy()
    lib().eo_divide_volume(den.size, pd(den), pd(vol))
    return den


def density_from_fixed(acc, fx, vol):
    den = np.zeros(acc.size)
    lib().eo_density_from_fixed(acc.size, pi64(acc), 1.0 / fx, pd(vol), pd(den))
    return den


def charge_density(charges, dens):
    dens = np.ascontiguousarray(dens, dtype=np.float64)
    ch = np.ascontiguousarray(charges, dtype=np.float64)
    rho = np.zeros(dens.shape[1])
    lib().eo_charge_density(dens.shape[1], dens.shape[0], pd(ch), pd(dens), pd(rho))
    return rho


def fixed_scale_exponent(weight_bound, capacity):
    return lib().eo_fixed_scale_exponent(weight_bound, capacity)


def sor_box(g, phi, rho, max_it, tol, order="rb"):
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    l2 = C.c_double(0)
    it = C.c_int(0)
    f = lib().eo_sor_box_rb if order == "rb" else lib().eo_sor_box_lex
    conv = f(C.byref(g), pd(phi), pd(rho), max_it, tol, C.byref(l2), C.byref(it))
    return phi, bool(conv), l2.value, it.value


def residual_box(g, phi, rho):
    return lib().eo_residual_box(C.byref(g), pd(phi), pd(rho))


def objects(g, center, radius, phi_s, inlet=True):
    obj = np.zeros(g.nn, dtype=np.int32)
    phi = np.zeros(g.nn)
    if radius is not None:
        lib().eo_objects_sphere(C.byref(g), arr3(center), radius, phi_s, pi(obj), pd(phi))
    if inlet:
        lib().eo_objects_inlet(C.byref(g), pi(obj), pd(phi))
    return obj, phi


def neumann_targets(g, obj):
    t = np.zeros(g.nn, dtype=np.int32)
    lib().eo_neumann_targets(C.byref(g), pi(obj), pi(t))
    return t


def residual_sphere(g, phi, rho, obj, phi0, te0, n0):
    return lib().eo_residual_sphere(C.byref(g), pd(phi), pd(rho), pi(obj), phi0, te0, n0)


def gs_sphere(g, phi, rho, obj, phi0, te0, n0, max_it, tol, order="rb"):
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    l2 = C.c_double(0)
    it = C.c_int(0)
    if order == "rb":
        t = neumann_targets(g, obj)
        conv = lib().eo_sor_sphere_rb(C.byref(g), pd(phi), pd(rho), pi(obj), pi(t), phi0, te0, n0,
                                      max_it, tol, C.byref(l2), C.byref(it))
    else:
        conv = lib().eo_gs_sphere_lex(C.byref(g), pd(phi), pd(rho), pi(obj), phi0, te0, n0, max_it,
                                      tol, C.byref(l2), C.byref(it))
    return phi, bool(conv), l2.value, it.value


def qn(g, phi, rho, obj, phi0, te0, n0):
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    lib().eo_qn(C.byref(g), pd(phi), pd(rho), pi(obj), phi0, te0, n0)
    return phi


def newton_pcg(g, phi, rho, obj, phi0, te0, n0, nr_max=20, nr_tol=1e-6, pcg_max=10000,
               pcg_tol=1e-8):
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    t = neumann_targets(g, obj)
    a = C.c_int(0)
    b = C.c_int(0)
    conv = lib().eo_newton_pcg(C.byref(g), pd(phi), pd(rho), pi(obj), pi(t), phi0, te0, n0, nr_max,
                               nr_tol, pcg_max, pcg_tol, C.byref(a), C.byref(b))
    return phi, bool(conv), a.value, b.value


def newton_pcg_fallback(g, phi, rho, obj, phi0, te0, n0, nr_max, nr_tol, pcg_max, pcg_tol, gs_max, gs_tol,
                        early_stop=False):
    """Newton-PCG with the reference's Gauss-Seidel fallback after a failed
    inner PCG (and, with early_stop, the CUDA path's inner stop on the RMS of
    the preconditioned residual); returns (phi, converged, newton, pcg, gs
    sweeps)"""
    L = lib()
    f = L.eo_newton_pcg_fb
    f.restype = C.c_int
    f.argtypes = [C.POINTER(Grid), PD, PD, PI, PI, D, D, D, C.c_int, D, C.c_int, D, C.c_int, D, C.c_int, PI, PI,
                  PI]
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    t = neumann_targets(g, obj)
    a, b, c = C.c_int(0), C.c_int(0), C.c_int(0)
    conv = f(C.byref(g), pd(phi), pd(rho), pi(obj), pi(t), phi0, te0, n0, nr_max, nr_tol, pcg_max, pcg_tol, gs_max,
             gs_tol, 1 if early_stop else 0, C.byref(a), C.byref(b), C.byref(c))
    return phi, bool(conv), a.value, b.value, c.value


def efield(g, phi):
    ef = np.zeros((g.nn, 3))
    lib().eo_efield(C.byref(g), pd(np.ascontiguousarray(phi, dtype=np.float64)), pd(ef))
    return ef


def species_diag(P, mass):
    P = np.ascontiguousarray(P, dtype=np.float64)
    out = np.zeros(5)
    lib().eo_species_diag(pd(P), P.shape[1], P.shape[1], mass, pd(out))
    return out


def potential_energy(g, ef, vol):
    return lib().eo_potential_energy(C.byref(g), pd(np.ascontiguousarray(ef)), pd(vol))


def update_average(ave, inst, samples):
    ave = np.ascontiguousarray(ave, dtype=np.float64).copy()
    lib().eo_update_average(ave.size, pd(ave), pd(np.ascontiguousarray(inst)), samples)
    return ave


# ---------------------------------------------------------------- reference
def kv_write(path, d):
    with open(path, "wb") as f:
        for k, v in d.items():
            a = np.ascontiguousarray(np.asarray(v, dtype=np.float64).ravel())
            kb = k.encode()
            f.write(struct.pack("<i", len(kb)))
            f.write(kb)
            f.write(struct.pack("<q", a.size))
            f.write(a.tobytes())


def kv_read(path):
    out = {}
    with open(path, "rb") as f:
        data = f.read()
    off = 0
    while off < len(data):
        (ln,) = struct.unpack_from("<i", data, off)
        off += 4
        k = data[off:off + ln].decode()
        off += ln
        (cnt,) = struct.unpack_from("<q", data, off)
        off += 8
        out[k] = np.frombuffer(data, dtype=np.float64, count=cnt, offset=off).copy()
        off += 8 * cnt
    return out


def run_reference(binary, op, inputs):
    """Run one reference harness operation; returns its output records."""
    exe = build_ref.ref_binary(binary)
    with tempfile.TemporaryDirectory() as td:
        fi = os.path.join(td, "in.kv")
        fo = os.path.join(td, "out.kv")
        kv_write(fi, inputs)
        subprocess.run([exe, op, fi, fo], check=True, stdout=subprocess.DEVNULL,
                       stderr=subprocess.DEVNULL)
        return kv_read(fo)


# ---- the mixed particle form (the chosen GPU form), restated -------------------
class MixArgs(C.Structure):
    _fields_ = [("ni", C.c_int), ("nj", C.c_int), ("nk", C.c_int), ("qmdt", C.c_float),
                ("dtdh", C.c_float * 3), ("dh", C.c_float * 3), ("sx", C.c_float * 3), ("r2", C.c_float)]


def _sig_mixed(L):
    PF = C.POINTER(C.c_float)
    P32 = C.POINTER(C.c_int32)
    PU8 = C.POINTER(C.c_uint8)
    L.eo_mix_args_set.argtypes = [C.POINTER(MixArgs), C.POINTER(Grid), D, D, D, PD]
    L.eo_ef_to_f32.argtypes = [I64, PD, PF]
    L.eo_to_mixed.argtypes = [C.POINTER(Grid), PD, I64, I64, P32, PF, PF, I64]
    L.eo_from_mixed.argtypes = [C.POINTER(Grid), P32, PF, PF, I64, I64, D, PD, I64]
    L.eo_push_mixed.argtypes = [C.POINTER(MixArgs), PF, C.c_int, P32, PF, PF, I64, I64, PU8]
    L.eo_compact_mixed.restype = I64
    L.eo_compact_mixed.argtypes = [P32, PF, PF, I64, I64, PU8]
    L.eo_deposit_mixed.argtypes = [C.POINTER(Grid), P32, PF, I64, I64, PU8, PI64]


def _mlib():
    L = lib()
    if not getattr(L, "_mixed_sig", False):
        _sig_mixed(L)
        L._mixed_sig = True
    return L


def _pf(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _p32(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int32))


def _pu8(a):
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint8))


def mix_args(g, charge, mass, dt, sphere4=None):
    a = MixArgs()
    sph = None if sphere4 is None else np.ascontiguousarray(sphere4, dtype=np.float64)
    _mlib().eo_mix_args_set(C.byref(a), C.byref(g), charge, mass, dt, None if sph is None else pd(sph))
    return a


def ef_to_f32(ef):
    ef = np.ascontiguousarray(ef, dtype=np.float64).reshape(-1)
    nn = ef.size // 3
    out = np.zeros(4 * nn, dtype=np.float32)
    _mlib().eo_ef_to_f32(nn, pd(ef), _pf(out))
    return out


def to_mixed(g, P):
    """float64 block [7][n] -> (cell [n] int32, off [3][n] f32, vel [3][n] f32)"""
    P = np.ascontiguousarray(P, dtype=np.float64)
    n = P.shape[1]
    cell = np.zeros(n, dtype=np.int32)
    off = np.zeros((3, n), dtype=np.float32)
    vel = np.zeros((3, n), dtype=np.float32)
    _mlib().eo_to_mixed(C.byref(g), pd(P), n, n, _p32(cell), _pf(off), _pf(vel), n)
    return cell, off, vel


def from_mixed(g, cell, off, vel, mpw0):
    n = cell.size
    P = np.zeros((7, n))
    _mlib().eo_from_mixed(C.byref(g), _p32(np.ascontiguousarray(cell)), _pf(np.ascontiguousarray(off)),
                          _pf(np.ascontiguousarray(vel)), n, n, mpw0, pd(P), n)
    return P


def push_mixed(a, ef4, walls, cell, off, vel, compact=True):
    """One mixed push (walls 0 reflect, 1 absorb); with compact the dead are
    removed in the GPU's holes order.  Returns (cell, off, vel, dead)."""
    cell = np.ascontiguousarray(cell, dtype=np.int32).copy()
    off = np.ascontiguousarray(off, dtype=np.float32).copy()
    vel = np.ascontiguousarray(vel, dtype=np.float32).copy()
    n = cell.size
    dead = np.zeros(n, dtype=np.uint8)
    L = _mlib()
    L.eo_push_mixed(C.byref(a), _pf(np.ascontiguousarray(ef4, dtype=np.float32)), walls, _p32(cell), _pf(off),
                    _pf(vel), n, n, _pu8(dead))
    if not compact:
        return cell, off, vel, dead
    m = L.eo_compact_mixed(_p32(cell), _pf(off), _pf(vel), n, n, _pu8(dead))
    return cell[:m].copy(), np.ascontiguousarray(off[:, :m]), np.ascontiguousarray(vel[:, :m]), dead


def deposit_mixed(g, cell, off, skip=None):
    """int64 node sums of round(w * 2^23) per corner (counts of mpw0 * 2^-23)"""
    cell = np.ascontiguousarray(cell, dtype=np.int32)
    off = np.ascontiguousarray(off, dtype=np.float32)
    n = cell.size
    acc = np.zeros(g.nn, dtype=np.int64)
    sk = None if skip is None else _pu8(np.ascontiguousarray(skip, dtype=np.uint8))
    _mlib().eo_deposit_mixed(C.byref(g), _p32(cell), _pf(off), n, n, sk, pi64(acc))
    return acc


def chemistry_ionize_offsets(g, den_n, rho, ef, charge, mass, mpw0, rate, dt, u, max_new=200000):
    """eo_chemistry_ionize_ex: (new ions [7][m], their time left, uniforms
    used, each cell's first uniform in the reference's cell order)"""
    L = lib()
    f = L.eo_chemistry_ionize_ex
    f.restype = I64
    f.argtypes = [C.POINTER(Grid), PD, PD, PD, D, D, D, D, D, PD, I64, PD, PD, I64, PI64, PI64]
    den_n, rho, ef = (np.ascontiguousarray(a, dtype=np.float64) for a in (den_n, rho, ef))
    u = np.ascontiguousarray(u, dtype=np.float64)
    Q, qdt = np.zeros((7, max_new)), np.zeros(max_new)
    ncell = (g.ni - 1) * (g.nj - 1) * (g.nk - 1)
    off = np.zeros(ncell, dtype=np.int64)
    used = C.c_int64(0)
    m = f(C.byref(g), pd(den_n), pd(rho), pd(ef), charge, mass, mpw0, rate, dt, pd(Q), max_new, pd(qdt), pd(u),
          u.size, C.byref(used), pi64(off))
    assert m >= 0, "uniforms ran out or the buffer of new particles is full"
    return np.ascontiguousarray(Q[:, :m]), qdt[:m].copy(), used.value, off


def advance_ch4_ion_holes(g, ef, sphere, charge, mass, mpw0, dt, P, pdt, neutral, spherium, u, max_new=100000):
    """eo_advance_ch4_ion_ex with the CUDA path's removal order: (P, pdt,
    created [7][m], tags, their time left, uniforms used, each particle's
    first uniform)"""
    L = lib()
    f = L.eo_advance_ch4_ion_ex
    f.restype = I64
    f.argtypes = [C.POINTER(Grid), PD, PD, D, D, D, D, PD, I64, I64, PD, D, D, D, D, D, D, PD, I64,
                  C.POINTER(C.c_int32), PD, PI64, PD, I64, PI64, PI64, C.c_int]
    P = np.array(P, dtype=np.float64, order="C", copy=True)
    pdt = np.array(pdt, dtype=np.float64, copy=True)
    u = np.ascontiguousarray(u, dtype=np.float64)
    ef = np.ascontiguousarray(ef, dtype=np.float64)
    sph = np.array(list(sphere[:3]) + [sphere[3] ** 2], dtype=np.float64)
    n = P.shape[1]
    Q = np.zeros((7, max_new))
    tag = np.zeros(max_new, dtype=np.int32)
    qdt = np.zeros(max_new)
    off = np.zeros(max(n, 1), dtype=np.int64)
    m, used = C.c_int64(0), C.c_int64(0)
    npart = f(C.byref(g), pd(ef), pd(sph), charge, mass, mpw0, dt, pd(P), n, n, pd(pdt), neutral[0], neutral[1],
              neutral[2], spherium[0], spherium[1], spherium[2], pd(Q), max_new,
              tag.ctypes.data_as(C.POINTER(C.c_int32)), pd(qdt), C.byref(m), pd(u), u.size, C.byref(used), pi64(off),
              1)
    assert npart >= 0, "uniforms ran out or the buffer of new particles is full"
    k = m.value
    return (np.ascontiguousarray(P[:, :npart]), pdt[:npart].copy(), np.ascontiguousarray(Q[:, :k]), tag[:k].copy(),
            qdt[:k].copy(), used.value, off[:n].copy())
