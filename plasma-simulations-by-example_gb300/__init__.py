"""Python view of libespic, the GB300-native electrostatic PIC time step.

The product is the C-ABI shared library built from csrc/ (declared in
include/espic.h) and the C++ drop-in headers in shim/.  This module is a thin
ctypes harness over the same C-ABI, used by the tests and the benchmark.  It
has no compute of its own and no CPU path: if the library is missing or no GPU
is present, creating a World raises.

Class and method names follow the reference (World, Species, PotentialSolver,
ColdBeamSource / WarmBeamSource); see include/espic.h for the reference
interface each call replaces.
"""
import ctypes as C
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libespic.so")

OK, NOT_CONVERGED = 0, 1
FORM_FP64, FORM_MIXED = 0, 1
WALLS_REFLECT, WALLS_ABSORB = 0, 1
SOLVER_SOR, SOLVER_GS, SOLVER_PCG, SOLVER_QN = 0, 1, 2, 3
FIELD_PHI, FIELD_RHO, FIELD_NODE_VOL, FIELD_EF, FIELD_DEN, FIELD_DEN_AVE, FIELD_OBJECT_ID = range(7)
FIELD_VEL, FIELD_TEMP, FIELD_MPC, FIELD_MOMENTS = range(7, 11)
BEAM_COLD, BEAM_WARM, BEAM_ISOTROPIC, BEAM_MAXWELLIAN = range(4)
COUNT_RANDOM, COUNT_REMAINDER = 0, 1

QE, AMU, ME, K, EPS_0 = 1.602176565e-19, 1.660538921e-27, 9.10938215e-31, 1.380648e-23, 8.85418782e-12

_lib = None

PD = C.POINTER(C.c_double)
PI = C.POINTER(C.c_int)
I64 = C.c_int64
VP = C.c_void_p


class EspicError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("espic status %d: %s" % (code, msg))
        self.code = code


def build(force=False):
    from importlib import util
    spec = util.spec_from_file_location("_espic_build", os.path.join(PKG_DIR, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def _build_module():
    from importlib import util
    spec = util.spec_from_file_location("_espic_build", os.path.join(PKG_DIR, "build.py"))
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def build_shim(force=False):
    """libespic_shim.a: the drop-in World/Species/PotentialSolver classes."""
    return _build_module().build_shim(force=force)


def compile_drop_in(main_source, out, stdin_source=False):
    return _build_module().compile_drop_in(main_source, out, stdin_source)


def lib():
    """The loaded libespic.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise EspicError(-2, "libespic.so not built (run __graft_entry__.build())")
        L = C.CDLL(LIB_PATH)
        sigs = {
            "espic_last_error": [C.c_char_p, C.c_int],
            "espic_world_create": [C.c_int, C.c_int, C.c_int, PD, PD, C.POINTER(VP)],
            "espic_world_destroy": [VP],
            "espic_world_set_time": [VP, C.c_double, C.c_int],
            "espic_world_advance_time": [VP],
            "espic_world_get_time": [VP, PI, PD],
            "espic_world_add_sphere": [VP, PD, C.c_double, C.c_double],
            "espic_world_add_inlet": [VP],
            "espic_world_set_seed": [VP, C.c_uint64],
            "espic_world_sync": [VP],
            "espic_world_stream": [VP, C.POINTER(VP)],
            "espic_species_create": [VP, C.c_double, C.c_double, C.c_double, I64, C.c_int, C.c_int,
                                     C.c_double, PI],
            "espic_species_count": [VP, C.c_int, C.POINTER(I64)],
            "espic_species_add": [VP, C.c_int, PD, PD, PD, I64],
            "espic_species_set": [VP, C.c_int, PD, I64, I64],
            "espic_species_get": [VP, C.c_int, PD, I64, I64, C.POINTER(I64)],
            "espic_species_set_mixed": [VP, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), I64, I64],
            "espic_species_get_mixed": [VP, C.c_int, C.POINTER(C.c_int32), C.POINTER(C.c_float),
                                        C.POINTER(C.c_float), I64, I64, C.POINTER(I64)],
            "espic_species_load_box": [VP, C.c_int, PD, PD, C.c_double, I64, PD],
            "espic_species_load_box_qs": [VP, C.c_int, PD, PD, C.c_double, PI],
            "espic_species_load_box_thermal": [VP, C.c_int, PD, PD, C.c_double, I64, PD, C.c_double, PD],
            "espic_push": [VP, C.c_int, C.c_int],
            "espic_deposit": [VP, C.c_int],
            "espic_charge_density": [VP],
            "espic_sort": [VP, C.c_int],
            "espic_source_create": [VP, C.c_int, C.c_double, C.c_double, C.c_double, PI],
            "espic_source_sample": [VP, C.c_int],
            "espic_source_sample_uniforms": [VP, C.c_int, PD, I64, C.POINTER(I64)],
            "espic_source_set_mode": [VP, C.c_int, C.c_int, C.c_int],
            "espic_solver_set": [VP, C.c_int, C.c_int, C.c_double],
            "espic_solver_set_reference": [VP, C.c_double, C.c_double, C.c_double],
            "espic_solver_set_newton": [VP, C.c_int, C.c_double, C.c_int, C.c_double, C.c_int],
            "espic_solver_set_multigrid": [VP, C.c_int, C.c_double],
            "espic_solver_set_launch": [VP, C.c_int],
            "espic_solver_set_coarse": [VP, I64],
            "espic_solver_set_dense": [VP, I64],
            "espic_solver_set_predictor": [VP, C.c_int],
            "espic_solver_set_fallback": [VP, C.c_int],
            "espic_solver_status": [VP, PI, PI, PI, PI, PD],
            "espic_solve": [VP, PI, PI, PD],
            "espic_efield": [VP],
            "espic_species_diag": [VP, C.c_int, PD],
            "espic_dsmc_enable": [VP, C.c_int, PD, C.c_double],
            "espic_dsmc_apply": [VP, C.c_int, C.c_double, PD, I64, C.POINTER(C.c_int64)],
            "espic_dsmc_status": [VP, C.c_int, PD, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
            "espic_sample_moments": [VP, C.c_int],
            "espic_gas_properties": [VP, C.c_int],
            "espic_clear_samples": [VP, C.c_int],
            "espic_compute_mpc": [VP, C.c_int],
            "espic_mcc_cex": [VP, C.c_int, C.c_int, C.c_double, PD, I64, C.POINTER(C.c_int64),
                              C.POINTER(C.c_int64)],
            "espic_advance_ch4": [VP, C.c_int, PD, PD, I64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
            "espic_advance_ch4_ions": [VP, C.c_int, C.c_int, C.c_int, PD, PD, I64, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int64)],
            "espic_chemistry_ionize": [VP, C.c_int, C.c_int, C.c_double, C.c_double, PD, I64,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int64)],
            "espic_potential_energy": [VP, PD],
            "espic_diag_row": [VP, PD, C.c_int],
            "espic_update_average": [VP, C.c_int],
            "espic_steady_state": [VP, PI],
            "espic_field_read": [VP, C.c_int, C.c_int, PD, I64],
            "espic_field_write": [VP, C.c_int, C.c_int, PD, I64],
            "espic_step": [VP, C.c_int, PD, C.c_int],
            "espic_profile": [VP, C.c_int],
            "espic_profile_read": [VP, PD, C.POINTER(I64), C.POINTER(I64)],
            "espic_solver_totals": [VP, C.POINTER(I64), C.POINTER(I64), C.POINTER(I64)],
            "espic_snapshot_begin": [VP, C.POINTER(I64)],
            "espic_snapshot_wait": [VP, I64, C.POINTER(PD), C.POINTER(I64)],
            "espic_ensemble_create": [C.c_int, PI, PD, PD, C.c_int, PD, PD, PD, C.POINTER(I64), C.c_double,
                                      C.POINTER(VP)],
            "espic_ensemble_set_seed": [VP, C.c_uint64],
            "espic_ensemble_set_box_ids": [VP, PI],
            "espic_partition_boxes": [C.c_int, PD, C.c_int, PI, PD],
            "espic_ensemble_set_particles": [VP, C.c_int, C.c_int, PD, I64, I64],
            "espic_ensemble_get_particles": [VP, C.c_int, C.c_int, PD, I64, I64, C.POINTER(I64)],
            "espic_ensemble_load_box": [VP, C.c_int, C.c_int, PD, PD, I64],
            "espic_ensemble_set_solver": [VP, C.c_int, C.c_double, C.c_double],
            "espic_ensemble_set_launch": [VP, C.c_int, C.c_int, C.c_int, C.c_int],
            "espic_ensemble_get_launch": [VP, PI, PI, PI, PI],
            "espic_ensemble_autotune": [VP, PI, PI, PI, PD, PD],
            "espic_ensemble_prepare": [VP],
            "espic_ensemble_step": [VP, C.c_int],
            "espic_ensemble_step_direct": [VP, C.c_int],
            "espic_ensemble_sync": [VP],
            "espic_ensemble_launches": [VP, C.POINTER(I64)],
            "espic_ensemble_steps_taken": [VP, C.POINTER(I64)],
            "espic_ensemble_status": [VP, PI, PI, PD],
            "espic_ensemble_read": [VP, C.c_int, C.c_int, C.c_int, PD],
            "espic_ensemble_diag": [VP, PD],
            "espic_diff_create": [VP, C.c_int, C.c_double, C.c_double, C.c_double, I64, C.c_double, C.c_double,
                                  C.c_double, C.c_double, C.c_double, C.c_int, C.POINTER(VP)],
            "espic_diff_set_state": [VP, PD, PD],
            "espic_diff_forward": [VP, C.c_double, C.c_int, PD],
            "espic_diff_backward": [VP, PD, PD, PD],
        }
        for name, args in sigs.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = C.c_int
        L.espic_ensemble_destroy.argtypes = [VP]
        L.espic_ensemble_destroy.restype = None
        L.espic_ensemble_stream.argtypes = [VP]
        L.espic_ensemble_stream.restype = VP
        L.espic_diff_destroy.argtypes = [VP]
        L.espic_diff_destroy.restype = None
        _lib = L
    return _lib


def last_error():
    buf = C.create_string_buffer(512)
    lib().espic_last_error(buf, 512)
    return buf.value.decode()


def check(rc, allow=(OK,)):
    if rc not in allow:
        raise EspicError(rc, last_error())
    return rc


def _pd(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(PD)


def _d3(v):
    return (C.c_double * 3)(*[float(x) for x in v])


class World:
    """World (ch2/World.h:38-110, ch3/ver2/World.h:38-147) on the GPU."""

    def __init__(self, ni, nj, nk, x0, xm):
        h = VP()
        check(lib().espic_world_create(ni, nj, nk, _d3(x0), _d3(xm), C.byref(h)))
        self.h = h
        self.ni, self.nj, self.nk = ni, nj, nk
        self.nn = ni * nj * nk
        self.x0 = np.array(x0, dtype=float)
        self.xm = np.array(xm, dtype=float)
        self.dh = (self.xm - self.x0) / (np.array([ni, nj, nk]) - 1)
        self.species = []

    def close(self):
        if getattr(self, "h", None):
            lib().espic_world_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # World API
    def setTime(self, dt, num_ts):
        self.dt = dt
        check(lib().espic_world_set_time(self.h, dt, num_ts))

    def advanceTime(self):
        return bool(lib().espic_world_advance_time(self.h))

    def addSphere(self, center, radius, phi_sphere):
        check(lib().espic_world_add_sphere(self.h, _d3(center), radius, phi_sphere))

    def addInlet(self):
        check(lib().espic_world_add_inlet(self.h))

    def set_seed(self, seed):
        check(lib().espic_world_set_seed(self.h, seed))

    def sync(self):
        check(lib().espic_world_sync(self.h))

    def stream_handle(self):
        """The raw cudaStream_t of this world (for events on its stream)."""
        v = VP()
        check(lib().espic_world_stream(self.h, C.byref(v)))
        return v.value

    def computeChargeDensity(self):
        check(lib().espic_charge_density(self.h))

    def getPE(self):
        v = C.c_double()
        check(lib().espic_potential_energy(self.h, C.byref(v)))
        return v.value

    def steadyState(self):
        v = C.c_int()
        check(lib().espic_steady_state(self.h, C.byref(v)))
        return bool(v.value)

    def diag_row(self):
        row = np.zeros(6 * len(self.species) + 1)
        check(lib().espic_diag_row(self.h, _pd(row), row.size))
        return row

    def step(self, sort_every=0, row=None):
        if row is None:
            check(lib().espic_step(self.h, sort_every, None, 0))
            return None
        check(lib().espic_step(self.h, sort_every, _pd(row), row.size))
        return row

    # measurement
    PHASES = ("inject", "sort", "push", "compact", "density", "solve", "efield", "diag")

    def profile(self, enable=True):
        check(lib().espic_profile(self.h, 1 if enable else 0))

    def profile_read(self):
        ms = np.zeros(8)
        cnt = (I64 * 8)()
        nl = I64()
        check(lib().espic_profile_read(self.h, _pd(ms), cnt, C.byref(nl)))
        return {p: (ms[i], cnt[i]) for i, p in enumerate(self.PHASES)}, nl.value

    def launches(self):
        nl = I64()
        check(lib().espic_profile_read(self.h, None, None, C.byref(nl)))
        return nl.value

    def snapshot_begin(self):
        """Queue an output snapshot (object_id, node_vol, phi, rho, den and
        den_ave per species, ef) and return its ticket."""
        t = I64()
        check(lib().espic_snapshot_begin(self.h, C.byref(t)))
        return t.value

    def snapshot_wait(self, ticket):
        """The snapshot's fields as a dict of numpy copies."""
        ptr, cnt = PD(), I64()
        check(lib().espic_snapshot_wait(self.h, ticket, C.byref(ptr), C.byref(cnt)))
        a = np.ctypeslib.as_array(ptr, shape=(cnt.value,)).copy()
        nn = self.nn
        ns = (cnt.value // nn - 7) // 2
        out = {"object_id": a[:nn].astype(np.int32), "node_vol": a[nn:2 * nn], "phi": a[2 * nn:3 * nn],
               "rho": a[3 * nn:4 * nn]}
        for s in range(ns):
            out["den%d" % s] = a[(4 + s) * nn:(5 + s) * nn]
            out["den_ave%d" % s] = a[(4 + ns + s) * nn:(5 + ns + s) * nn]
        out["ef"] = a[(4 + 2 * ns) * nn:].reshape(nn, 3)
        return out

    def solver_totals(self):
        a, b, c = I64(), I64(), I64()
        check(lib().espic_solver_totals(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    # fields
    def read(self, field, sp=0):
        if field in (FIELD_EF, FIELD_VEL):
            out = np.zeros((self.nn, 3))
        elif field == FIELD_MPC:
            out = np.zeros((self.ni - 1) * (self.nj - 1) * (self.nk - 1))
        elif field == FIELD_MOMENTS:
            out = np.zeros((7, self.nn))
        else:
            out = np.zeros(self.nn)
        check(lib().espic_field_read(self.h, field, sp, _pd(out), out.size))
        return out

    def write(self, field, data, sp=0):
        a = np.ascontiguousarray(data, dtype=np.float64)
        check(lib().espic_field_write(self.h, field, sp, _pd(a), a.size))

    @property
    def phi(self):
        return self.read(FIELD_PHI)

    @property
    def rho(self):
        return self.read(FIELD_RHO)

    @property
    def ef(self):
        return self.read(FIELD_EF)

    @property
    def node_vol(self):
        return self.read(FIELD_NODE_VOL)

    @property
    def object_id(self):
        return self.read(FIELD_OBJECT_ID).astype(np.int32)


class Species:
    """Species (ch2/Species.h:22-65, ch3/ver2/Species.h:22-72) on the GPU."""

    def __init__(self, world, name, mass, charge, mpw0=0.0, capacity=1 << 20, form=FORM_FP64,
                 walls=WALLS_REFLECT, weight_bound=0.0):
        sid = C.c_int()
        check(lib().espic_species_create(world.h, mass, charge, mpw0, int(capacity), form, walls,
                                         weight_bound, C.byref(sid)))
        self.world, self.name, self.mass, self.charge, self.mpw0 = world, name, mass, charge, mpw0
        self.id = sid.value
        self.form = form
        self.capacity = capacity
        world.species.append(self)

    def getNp(self):
        n = I64()
        check(lib().espic_species_count(self.world.h, self.id, C.byref(n)))
        return n.value

    def addParticles(self, pos3, vel3, mpw=None):
        pos3 = np.ascontiguousarray(pos3, dtype=np.float64)
        vel3 = np.ascontiguousarray(vel3, dtype=np.float64)
        w = None if mpw is None else np.ascontiguousarray(mpw, dtype=np.float64)
        check(lib().espic_species_add(self.world.h, self.id, _pd(pos3), _pd(vel3), _pd(w),
                                      pos3.shape[0]))

    def set_particles(self, P):
        P = np.ascontiguousarray(P, dtype=np.float64)
        check(lib().espic_species_set(self.world.h, self.id, _pd(P), P.shape[1], P.shape[1]))

    def particles(self):
        n = self.getNp()
        P = np.zeros((7, max(n, 1)))
        m = I64()
        check(lib().espic_species_get(self.world.h, self.id, _pd(P), P.shape[1], P.shape[1],
                                      C.byref(m)))
        return np.ascontiguousarray(P[:, :m.value])

    def set_mixed(self, cell, off, vel):
        """the mixed form's own state: cell keys [n] int32, offsets and
        velocities [3][n] float32 (no conversion)"""
        cell = np.ascontiguousarray(cell, dtype=np.int32)
        off = np.ascontiguousarray(off, dtype=np.float32)
        vel = np.ascontiguousarray(vel, dtype=np.float32)
        n = cell.size
        check(lib().espic_species_set_mixed(self.world.h, self.id, cell.ctypes.data_as(C.POINTER(C.c_int32)),
                                            off.ctypes.data_as(C.POINTER(C.c_float)),
                                            vel.ctypes.data_as(C.POINTER(C.c_float)), n, n))

    def get_mixed(self):
        """(cell [n] int32, off [3][n] float32, vel [3][n] float32)"""
        m = I64()
        check(lib().espic_species_get_mixed(self.world.h, self.id, None, None, None, 0, 0, C.byref(m)))
        n = max(m.value, 1)
        cell = np.zeros(n, dtype=np.int32)
        off = np.zeros((3, n), dtype=np.float32)
        vel = np.zeros((3, n), dtype=np.float32)
        check(lib().espic_species_get_mixed(self.world.h, self.id, cell.ctypes.data_as(C.POINTER(C.c_int32)),
                                            off.ctypes.data_as(C.POINTER(C.c_float)),
                                            vel.ctypes.data_as(C.POINTER(C.c_float)), n, n, C.byref(m)))
        k = m.value
        return cell[:k].copy(), np.ascontiguousarray(off[:, :k]), np.ascontiguousarray(vel[:, :k])

    def loadParticlesBox(self, x1, x2, num_den, num_mp, u=None):
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        check(lib().espic_species_load_box(self.world.h, self.id, _d3(x1), _d3(x2), num_den,
                                           int(num_mp), _pd(u)))

    def loadParticlesBoxThermal(self, x1, x2, mpw, num_mp, v_drift, temp, u=None):
        """num_mp particles of weight mpw (0: mpw0) with a drifting Maxwellian."""
        u = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        check(lib().espic_species_load_box_thermal(self.world.h, self.id, _d3(x1), _d3(x2), mpw,
                                                   int(num_mp), _d3(v_drift), temp, _pd(u)))

    def loadParticlesBoxQS(self, x1, x2, num_den, num_mp):
        nm = (C.c_int * 3)(*[int(x) for x in num_mp])
        check(lib().espic_species_load_box_qs(self.world.h, self.id, _d3(x1), _d3(x2), num_den, nm))

    def advance(self, deposit=False):
        check(lib().espic_push(self.world.h, self.id, 1 if deposit else 0))

    def computeNumberDensity(self):
        check(lib().espic_deposit(self.world.h, self.id))

    def sort(self):
        check(lib().espic_sort(self.world.h, self.id))

    def diag(self):
        out = np.zeros(5)
        check(lib().espic_species_diag(self.world.h, self.id, _pd(out)))
        return out

    # DSMC_MEX, ch4/Collisions.h:51-75 (float64 form)
    def enable_dsmc(self, c=None, sigma_cr_max=1e-14):
        """Neutral-neutral collisions of this species (the reference's VHS
        parameters when c is None)."""
        cc = None if c is None else np.ascontiguousarray(c, dtype=np.float64)
        check(lib().espic_dsmc_enable(self.world.h, self.id, None if cc is None else _pd(cc), sigma_cr_max))

    def dsmc(self, dt, u=None, cell_off=None):
        """DSMC_MEX::apply(dt); with u and cell_off the uniforms are replayed
        (cell c starts at u[cell_off[c]])."""
        if u is None:
            check(lib().espic_dsmc_apply(self.world.h, self.id, dt, None, 0, None))
            return
        uu = np.ascontiguousarray(u, dtype=np.float64)
        off = np.ascontiguousarray(cell_off, dtype=np.int64)
        check(lib().espic_dsmc_apply(self.world.h, self.id, dt, _pd(uu), uu.size,
                                     off.ctypes.data_as(C.POINTER(C.c_int64))))

    def dsmc_status(self):
        """(sigma_cr_max, collisions of the last call, collisions of all calls)"""
        smax = C.c_double()
        last, total = C.c_int64(), C.c_int64()
        check(lib().espic_dsmc_status(self.world.h, self.id, C.byref(smax), C.byref(last), C.byref(total)))
        return smax.value, last.value, total.value

    def advance_ch4(self, pdt=None, u=None, p_off=None, count=False):
        """Species::advance(neutrals, spherium) of a neutral species
        (ch4/Species.cpp:8-100); pdt: each particle's time left (default: a
        dt for particles appended since the last call); u, p_off: replayed
        uniforms; count=True (or replay) waits and returns the bounces."""
        b = C.c_int64(0)
        pb = C.byref(b) if (count or u is not None or pdt is not None) else None
        pp = None
        if pdt is not None:
            pdt = np.ascontiguousarray(pdt, dtype=np.float64)
            pp = _pd(pdt)
        if u is None:
            check(lib().espic_advance_ch4(self.world.h, self.id, pp, None, 0, None, pb))
        else:
            uu = np.ascontiguousarray(u, dtype=np.float64)
            off = np.ascontiguousarray(p_off, dtype=np.int64)
            check(lib().espic_advance_ch4(self.world.h, self.id, pp, _pd(uu), uu.size,
                                          off.ctypes.data_as(C.POINTER(C.c_int64)), pb))
        return b.value if pb is not None else None

    def advance_ch4_ions(self, neutrals, spherium=None, pdt=None, u=None, p_off=None):
        """Species::advance(neutrals, spherium) of a charged species (ch4's
        ion branch, ch4/Species.cpp:8-91): ions striking the sphere are
        removed and create particles in `neutrals` and `spherium` (default:
        `neutrals`, as ch4/Main.cpp:81 calls it).  pdt, u, p_off as
        advance_ch4.  Waits; returns the number of strikes."""
        spherium = neutrals if spherium is None else spherium
        b = C.c_int64(0)
        pp = None
        if pdt is not None:
            pdt = np.ascontiguousarray(pdt, dtype=np.float64)
            pp = _pd(pdt)
        if u is None:
            check(lib().espic_advance_ch4_ions(self.world.h, self.id, neutrals.id, spherium.id, pp, None, 0,
                                               None, C.byref(b)))
        else:
            uu = np.ascontiguousarray(u, dtype=np.float64)
            off = np.ascontiguousarray(p_off, dtype=np.int64)
            check(lib().espic_advance_ch4_ions(self.world.h, self.id, neutrals.id, spherium.id, pp, _pd(uu),
                                               uu.size, off.ctypes.data_as(C.POINTER(C.c_int64)), C.byref(b)))
        return b.value

    # ch4 species moments (ch4/Species.cpp:191-240, float64 form)
    def sampleMoments(self):
        check(lib().espic_sample_moments(self.world.h, self.id))

    def computeGasProperties(self):
        check(lib().espic_gas_properties(self.world.h, self.id))

    def clearSamples(self):
        check(lib().espic_clear_samples(self.world.h, self.id))

    def computeMPC(self):
        check(lib().espic_compute_mpc(self.world.h, self.id))

    @property
    def vel(self):
        """stream velocity [nn][3] (computeGasProperties)"""
        return self.world.read(FIELD_VEL, self.id)

    @property
    def T(self):
        return self.world.read(FIELD_TEMP, self.id)

    @property
    def mpc(self):
        return self.world.read(FIELD_MPC, self.id)

    @property
    def moments(self):
        """sampled sums [7][nn]: n, nu, nv, nw, nuu, nvv, nww"""
        return self.world.read(FIELD_MOMENTS, self.id)

    def updateAverages(self):
        check(lib().espic_update_average(self.world.h, self.id))

    @property
    def den(self):
        return self.world.read(FIELD_DEN, self.id)

    @property
    def den_ave(self):
        return self.world.read(FIELD_DEN_AVE, self.id)


class MCC_CEX:
    """MCC_CEX(source, target, world) (ch4/Collisions.h:40-50): source
    particles collide with the target gas (its den and vel fields)."""

    def __init__(self, source, target, world=None):
        self.source, self.target = source, target
        self.world = world or source.world
        self.last = None

    def apply(self, dt, u=None, p_off=None, count=False):
        """MCC_CEX::apply(dt); with u and p_off the uniforms are replayed
        (particle p draws u[p_off[p]]); count=True waits and returns the
        number of colliding particles."""
        n = C.c_int64(0)
        pn = C.byref(n) if (count or u is not None) else None
        if u is None:
            check(lib().espic_mcc_cex(self.world.h, self.source.id, self.target.id, dt, None, 0, None, pn))
        else:
            uu = np.ascontiguousarray(u, dtype=np.float64)
            off = np.ascontiguousarray(p_off, dtype=np.int64)
            check(lib().espic_mcc_cex(self.world.h, self.source.id, self.target.id, dt, _pd(uu), uu.size,
                                      off.ctypes.data_as(C.POINTER(C.c_int64)), pn))
        self.last = n.value if pn is not None else None
        return self.last


class ChemistryIonize:
    """ChemistryIonize(neutrals, ions, world, rate) (ch4/Collisions.h:76-86):
    ions created at rate n_a n_e per cell (ch4/Collisions.cpp:10-31)."""

    def __init__(self, neutrals, ions, world=None, rate=0.0):
        self.neutrals, self.ions = neutrals, ions
        self.world = world or ions.world
        self.rate = float(rate)
        self.last = None

    def apply(self, dt, u=None, cell_off=None):
        """ChemistryIonize::apply(dt); with u and cell_off the uniforms are
        replayed (cell c, in the reference's loop order, draws
        u[cell_off[c]]).  Waits; returns the number of ions added."""
        n = C.c_int64(0)
        if u is None:
            check(lib().espic_chemistry_ionize(self.world.h, self.neutrals.id, self.ions.id, self.rate, dt, None, 0,
                                               None, C.byref(n)))
        else:
            uu = np.ascontiguousarray(u, dtype=np.float64)
            off = np.ascontiguousarray(cell_off, dtype=np.int64)
            check(lib().espic_chemistry_ionize(self.world.h, self.neutrals.id, self.ions.id, self.rate, dt,
                                               _pd(uu), uu.size, off.ctypes.data_as(C.POINTER(C.c_int64)),
                                               C.byref(n)))
        self.last = n.value
        return self.last


class BeamSource:
    """ColdBeamSource (temp = 0, ch3/ver2/Source.h:8-21) and WarmBeamSource
    (ch4/Source.h:32-46) on the z = x0 face."""

    def __init__(self, species, v_drift, den, temp=0.0):
        sid = C.c_int()
        check(lib().espic_source_create(species.world.h, species.id, v_drift, den, temp,
                                        C.byref(sid)))
        self.world = species.world
        self.id = sid.value
        self.temp = temp

    def set_mode(self, velocity_mode, count_mode=COUNT_RANDOM):
        """BEAM_COLD / BEAM_WARM (ch4) / BEAM_ISOTROPIC (ch9/MPI) /
        BEAM_MAXWELLIAN velocities; COUNT_RANDOM or COUNT_REMAINDER (ch9/MPI)."""
        check(lib().espic_source_set_mode(self.world.h, self.id, velocity_mode, count_mode))

    def sample(self, u=None):
        if u is None:
            check(lib().espic_source_sample(self.world.h, self.id))
            return None
        u = np.ascontiguousarray(u, dtype=np.float64)
        used = I64()
        check(lib().espic_source_sample_uniforms(self.world.h, self.id, _pd(u), u.size,
                                                 C.byref(used)))
        return used.value


class PotentialSolver:
    """PotentialSolver (ch2/PotentialSolver.h:6-23, ch3/ver2/PotentialSolver.h:42-104)."""

    def __init__(self, world, kind=SOLVER_SOR, max_it=10000, tol=1e-4):
        self.world = world
        check(lib().espic_solver_set(world.h, kind, max_it, tol))

    def setReferenceValues(self, phi0, te0, n0):
        check(lib().espic_solver_set_reference(self.world.h, phi0, te0, n0))

    def setNewton(self, nr_max=20, nr_tol=1e-3, pcg_max=10000, pcg_tol=1e-6, fp32_inner=False):
        check(lib().espic_solver_set_newton(self.world.h, nr_max, nr_tol, pcg_max, pcg_tol,
                                            1 if fp32_inner else 0))

    def setMultigrid(self, levels=12, scale=1.6):
        """levels = 0 selects the Jacobi preconditioner."""
        check(lib().espic_solver_set_multigrid(self.world.h, levels, scale))

    def setLaunch(self, max_blocks=0):
        check(lib().espic_solver_set_launch(self.world.h, max_blocks))

    def setFallback(self, enable=True):
        """Gauss-Seidel after an inner PCG that fails (the reference's
        fallback, ch3/ver2/PotentialSolver.cpp:270-271); on by default."""
        check(lib().espic_solver_set_fallback(self.world.h, 1 if enable else 0))

    def status(self):
        """(converged, iterations, inner iterations, fallback sweeps, norm) of
        the last solve"""
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        r = C.c_double()
        check(lib().espic_solver_status(self.world.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d), C.byref(r)))
        return bool(a.value), b.value, c.value, d.value, r.value

    def setPredictor(self, enable=True):
        """Start Newton solves of consecutive steps from 2 phi^n - phi^(n-1)
        (the float-inner solve, after three consecutive solves, from
        3 phi^n - 3 phi^(n-1) + phi^(n-2))."""
        check(lib().espic_solver_set_predictor(self.world.h, 1 if enable else 0))

    def setCoarse(self, block_nodes):
        """Multigrid levels with fewer nodes than this run on one block."""
        check(lib().espic_solver_set_coarse(self.world.h, int(block_nodes)))

    def setDense(self, max_nodes):
        """The first multigrid level with at most max_nodes nodes is the
        coarsest, solved by its dense inverse (0: smoothing sweeps)."""
        check(lib().espic_solver_set_dense(self.world.h, int(max_nodes)))

    def solve(self, wait=True):
        """Returns (converged, iterations, inner_iterations, residual)."""
        if not wait:
            check(lib().espic_solve(self.world.h, None, None, None))
            return None
        it, inner, res = C.c_int(), C.c_int(), C.c_double()
        rc = check(lib().espic_solve(self.world.h, C.byref(it), C.byref(inner), C.byref(res)),
                   allow=(OK, NOT_CONVERGED))
        return rc == OK, it.value, inner.value, res.value

    def computeEF(self):
        check(lib().espic_efield(self.world.h))


def partition_boxes(work, nparts):
    """Owner part of every box (largest work first, each to the least loaded
    part; the same on every rank) and the work of each part."""
    work = np.ascontiguousarray(work, dtype=np.float64)
    owner = np.zeros(max(work.size, 1), dtype=np.int32)
    load = np.zeros(nparts)
    check(lib().espic_partition_boxes(work.size, _pd(work), nparts, owner.ctypes.data_as(PI), _pd(load)))
    return owner[:work.size].copy(), load


def ensemble_work(nodes, particles, node_weight=14.0):
    """Work of a box step: its particles plus node_weight per node (the SOR
    sweeps cost about 14 particle pushes per node on a GB300)."""
    nodes = np.asarray(nodes).reshape(-1, 3)
    return np.asarray(particles, dtype=np.float64) + node_weight * np.prod(nodes, axis=1).astype(np.float64)


class Ensemble:
    """A batched ensemble of independent ch2 grounded boxes (ch2/Main.cpp:14-75
    per member): per-box node counts and extents, per (box, species) weights
    and capacities, stepped together on one GPU (see espic_ensemble_* in
    include/espic.h)."""

    def __init__(self, nodes, x0, xm, mass, charge, mpw0, capacity, dt):
        nodes = np.ascontiguousarray(nodes, dtype=np.int32).reshape(-1, 3)
        nbox = nodes.shape[0]
        x0 = np.ascontiguousarray(np.broadcast_to(np.asarray(x0, dtype=np.float64), (nbox, 3)))
        xm = np.ascontiguousarray(np.broadcast_to(np.asarray(xm, dtype=np.float64), (nbox, 3)))
        mass = np.ascontiguousarray(mass, dtype=np.float64)
        charge = np.ascontiguousarray(charge, dtype=np.float64)
        nsp = mass.size
        mpw0 = np.ascontiguousarray(np.broadcast_to(np.asarray(mpw0, dtype=np.float64), (nbox, nsp)))
        capacity = np.ascontiguousarray(np.broadcast_to(np.asarray(capacity, dtype=np.int64), (nbox, nsp)))
        h = VP()
        check(lib().espic_ensemble_create(nbox, nodes.ctypes.data_as(PI), _pd(x0), _pd(xm), nsp, _pd(mass),
                                          _pd(charge), _pd(mpw0), capacity.ctypes.data_as(C.POINTER(I64)), dt,
                                          C.byref(h)))
        self.h = h
        self.nodes, self.x0, self.xm = nodes, x0, xm
        self.nbox, self.nsp = nbox, nsp
        self.mass, self.charge, self.mpw0 = mass, charge, mpw0

    def set_box_ids(self, ids):
        """ids of these boxes in a larger ensemble (they key the boxes' random
        streams); None restores the box index"""
        if ids is None:
            check(lib().espic_ensemble_set_box_ids(self.h, None))
            return
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        assert ids.size == self.nbox
        check(lib().espic_ensemble_set_box_ids(self.h, ids.ctypes.data_as(PI)))

    def close(self):
        if self.h:
            lib().espic_ensemble_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_seed(self, seed):
        check(lib().espic_ensemble_set_seed(self.h, seed))

    def set_particles(self, box, sp, P):
        P = np.ascontiguousarray(P, dtype=np.float64)
        check(lib().espic_ensemble_set_particles(self.h, box, sp, _pd(P), P.shape[1], P.shape[1]))

    def particles(self, box, sp, cap=None):
        n = I64()
        check(lib().espic_ensemble_get_particles(self.h, box, sp, None, 0, 0, C.byref(n)))
        P = np.zeros((7, max(n.value, 1)))
        check(lib().espic_ensemble_get_particles(self.h, box, sp, _pd(P), P.shape[1], P.shape[1],
                                                 C.byref(n)))
        return np.ascontiguousarray(P[:, :n.value])

    def load_box(self, box, sp, x1, x2, num_mp):
        check(lib().espic_ensemble_load_box(self.h, box, sp, _d3(x1), _d3(x2), int(num_mp)))

    def set_solver(self, max_it=10000, tol=1e-4, omega=0.0):
        check(lib().espic_ensemble_set_solver(self.h, max_it, tol, omega))

    def set_launch(self, chunk, push_threads, solve_threads, cluster=8):
        check(lib().espic_ensemble_set_launch(self.h, chunk, push_threads, solve_threads, cluster))

    def get_launch(self):
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(lib().espic_ensemble_get_launch(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(d)))
        return a.value, b.value, c.value, d.value

    def autotune(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        pm, sm = C.c_double(), C.c_double()
        check(lib().espic_ensemble_autotune(self.h, C.byref(a), C.byref(b), C.byref(c), C.byref(pm),
                                            C.byref(sm)))
        cl = C.c_int()
        check(lib().espic_ensemble_get_launch(self.h, None, None, None, C.byref(cl)))
        return dict(chunk=a.value, push_threads=b.value, solve_threads=c.value, cluster=cl.value,
                    push_ms=pm.value, solve_ms=sm.value)

    def prepare(self):
        check(lib().espic_ensemble_prepare(self.h))

    def step(self, nsteps=1, graph=True):
        f = lib().espic_ensemble_step if graph else lib().espic_ensemble_step_direct
        check(f(self.h, nsteps))

    def sync(self):
        check(lib().espic_ensemble_sync(self.h))

    def stream_handle(self):
        return lib().espic_ensemble_stream(self.h)

    def launches(self):
        n = I64()
        check(lib().espic_ensemble_launches(self.h, C.byref(n)))
        return n.value

    def status(self):
        it = np.zeros(self.nbox, dtype=np.int32)
        cv = np.zeros(self.nbox, dtype=np.int32)
        res = np.zeros(self.nbox)
        check(lib().espic_ensemble_status(self.h, it.ctypes.data_as(PI), cv.ctypes.data_as(PI), _pd(res)))
        return it, cv.astype(bool), res

    def read(self, box, field, sp=0):
        nn = int(np.prod(self.nodes[box]))
        out = np.zeros(nn * (3 if field == FIELD_EF else 1))
        check(lib().espic_ensemble_read(self.h, box, field, sp, _pd(out)))
        return out.reshape(nn, 3) if field == FIELD_EF else out

    def diag(self):
        out = np.zeros((self.nbox, self.nsp + 1))
        check(lib().espic_ensemble_diag(self.h, _pd(out)))
        return out


class DiffRun:
    """Differentiable sphere run (espic_diff_* in include/espic.h): one ion
    species in `world` (sphere, inlet, reference values and Newton controls
    set on the world), no injection, C1 absorption over a layer of thickness
    delta.  Loss = alpha * final field energy + beta * ions in the wake box
    (nodes with z in wake_z).  precision: "fp64" or "fp32"."""

    def __init__(self, world, n, mass, charge, mpw0, delta, wake_z, alpha=1.0, beta=1.0, checkpoint_every=20,
                 precision="fp64"):
        h = VP()
        check(lib().espic_diff_create(world.h, 0 if precision == "fp64" else 1, mass, charge, mpw0, int(n), delta,
                                      wake_z[0], wake_z[1], alpha, beta, checkpoint_every, C.byref(h)))
        self.h, self.world, self.n = h, world, int(n)

    def close(self):
        if self.h:
            lib().espic_diff_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, x, v):
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(3, self.n)
        v = np.ascontiguousarray(v, dtype=np.float64).reshape(3, self.n)
        check(lib().espic_diff_set_state(self.h, _pd(x), _pd(v)))

    def forward(self, phi_sphere, nsteps):
        loss = C.c_double()
        check(lib().espic_diff_forward(self.h, phi_sphere, int(nsteps), C.byref(loss)))
        return loss.value

    def backward(self):
        """(d loss / d phi_sphere, d loss / d x [3][n], d loss / d v [3][n])"""
        dps = C.c_double()
        dx = np.zeros((3, self.n))
        dv = np.zeros((3, self.n))
        check(lib().espic_diff_backward(self.h, C.byref(dps), _pd(dx), _pd(dv)))
        return dps.value, dx, dv


def sphere_run_loss(run, phi_sphere, x0, v0, nsteps):
    """The loss of a DiffRun as a differentiable torch function of the sphere
    potential (0-d tensor), the initial positions and velocities ([3, n]
    float64 tensors); backward() calls the adjoint kernels."""
    import torch

    class _SphereRun(torch.autograd.Function):
        @staticmethod
        def forward(ctx, ps, x, v):
            run.set_state(x.detach().cpu().numpy(), v.detach().cpu().numpy())
            loss = run.forward(float(ps), nsteps)
            ctx.dev = x.device
            return torch.tensor(loss, dtype=torch.float64, device=x.device)

        @staticmethod
        def backward(ctx, g):
            dps, dx, dv = run.backward()
            t = lambda a: torch.as_tensor(a, dtype=torch.float64, device=ctx.dev)
            return g * t(dps), g * t(dx), g * t(dv)

    return _SphereRun.apply(phi_sphere, x0, v0)
