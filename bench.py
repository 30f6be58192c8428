"""Benchmark of the ES-PIC time step on GB300 (one JSON line on stdout).

Workload (default, configuration 5): flow past a sphere on a
256x256x512-node grid over [-0.1,0.1]^2 x [0,0.4] m, sphere r = 0.04 m at
(0,0,0.15) held at -100 V, z = 0 inlet Dirichlet, other walls Neumann; O+
warm beam (7 km/s drift, T_i = 0.1 eV, n0 = 1e10 m^-3) with mpw0 = 0.32 so
that about 480M macroparticles fill the domain (~14.5 per cell); Boltzmann
electrons (n0 = 1e10, Te = 3 eV, phi0 = 0); dt = 1e-7 s; Newton-PCG to RMS
update 1e-6 V; tile sort every 10 steps.  The reference has no published
dataset: the run starts from a synthetic steady-state stand-in, 500M ions
loaded on the GPU uniformly over the domain with the beam's drifting
thermal velocities (seeded; those inside the sphere are absorbed by the
first push), followed by an initial solve.  --config sphere64 is the
reference's configuration 2 (64x64x128 nodes, ~4M ions, mpw0 = 40).

A step = inject + push/deposit (+ the sort every 10) + charge density + Newton-PCG
+ computeEF.  value = particle-steps/s of the mixed form (int32 cell + f32
offset + f32 velocity; float PCG under a Newton residual in double-float,
pairs of floats with ~48 significant bits), timed with
CUDA events on the library's own stream; the L2 is flushed between timed
steps (outside the events).  The plain FP64 form runs the same workload.
e2e = the same step through the C-ABI as a user drives it, with the step's
injection uniforms copied from pinned host memory and the diagnostics row
(Output::diagOutput columns) read back every step.

--impl reference times the CPU implementation of the path on this host's
cores (the C restatement in oracle/: threaded push + deposit as ch9/MT does,
serial Newton-PCG timed per iteration and scaled to the iteration count the
GPU needed at this state).

Other workloads (--config): sphere64 and sphere128 (the same step on
smaller grids), box21 (the ch2 box, FP64 form), ensemble512 (512 ch2 boxes
stepped together), diff32 (forward + adjoint of the sphere run), dsmc41
(one DSMC_MEX::apply over the 6.4M-atom ch4 neutral gas, with the ch4
moment sampling, MCC and neutral push timed beside it; its reference arm
runs the oracle's DSMC_MEX on the host).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s + Poisson ms/step, mixed vs FP64 on GB300 at phi rel err ≤1e-6"
QE, AMU, K = 1.602176565e-19, 1.660538921e-27, 1.380648e-23

CONFIGS = {
    "sphere64": dict(n=(64, 64, 128), x0=(-0.1, -0.1, 0.0), xm=(0.1, 0.1, 0.4), center=(0, 0, 0.15),
                     radius=0.05, phi_s=-100.0, np=4_000_000, mpw0=40.0, dt=1e-7, sort_every=20),
    "sphere256": dict(n=(256, 256, 512), x0=(-0.1, -0.1, 0.0), xm=(0.1, 0.1, 0.4), center=(0, 0, 0.15),
                      radius=0.04, phi_s=-100.0, np=500_000_000, mpw0=0.32, dt=1e-7, sort_every=10),
    # the 256x256x512 plasma on an eighth of the cells (the same ions per
    # cell): small enough for a full ncu capture of the push at that density
    "sphere128": dict(n=(128, 128, 256), x0=(-0.1, -0.1, 0.0), xm=(0.1, 0.1, 0.4), center=(0, 0, 0.15),
                      radius=0.04, phi_s=-100.0, np=60_000_000, mpw0=0.32 * 500 / 60, dt=1e-7, sort_every=20),
    # the reference's configuration 1: ch2 grounded box, FP64 plain form
    "box21": dict(n=(21, 21, 21), x0=(-0.1, -0.1, 0.0), xm=(0.1, 0.1, 0.2), np=90_000, dt=2e-10,
                  sort_every=0),
    # batched ensemble: 512 ch2 boxes with drawn sizes, counts and densities
    "ensemble512": dict(nbox=512, x0=(-0.1, -0.1, 0.0), xm=(0.1, 0.1, 0.2), dt=2e-10, seed=2024),
    # ch4 neutral gas (ch4/Main.cpp:21-58): O atoms at 2e20 m^-3, 1000 K,
    # 7 km/s along z, mpw0 1e12 on a 41x21x41-node box; a step is one
    # DSMC_MEX::apply (Bird's NTC pairs, VHS cross-section) over all atoms
    "dsmc41": dict(n=(41, 21, 41), x0=(-0.2, -0.1, 0.0), xm=(0.2, 0.1, 0.4), nda=2e20, temp=1000.0, mpw0=1e12,
                   dt=1e-7),
    # differentiable sphere run: gradients by the adjoint kernels
    "diff32": dict(n=(32, 32, 64), x0=(-0.1, -0.1, 0.0), xm=(0.1, 0.1, 0.3), center=(0, 0, 0.15), radius=0.05,
                   phi_s=-100.0, np=500_000, dt=1e-7, steps=400, checkpoint=20, wake=(0.2, 0.3)),
}
V_DRIFT, N0, TI_EV, TE, PHI0 = 7000.0, 1e10, 0.1, 3.0, 0.0
NR_TOL, PCG_TOL = 1e-6, 1e-4


def espic_module():
    import importlib
    return importlib.import_module("plasma-simulations-by-example_gb300")


def measured_traffic(workload, kernel, units):
    """DRAM bytes of one launch of `kernel` processing `units` (PCG iterations
    or particles), scaled from the ncu capture recorded in
    profiles/traffic.txt; None when there is none."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.split()
        if len(f) >= 4 and not f[0].startswith("#") and f[0] == workload and f[1] == kernel:
            return float(f[2]) / float(f[3]) * float(units)
    return None


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi clock samples during the timed region."""

    def __init__(self):
        self.samples = []
        self.proc = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for i, n in enumerate(names):
                if len(s) > 2 + i and s[2 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def synthetic_state(cfg, n, seed):
    """n ions uniform outside the sphere with drifting thermal velocities."""
    rng = np.random.default_rng(seed)
    x0, xm = np.array(cfg["x0"]), np.array(cfg["xm"])
    c, r = np.array(cfg["center"]), cfg["radius"]
    m = 16 * AMU
    vth = np.sqrt(K * TI_EV * QE / K / m)
    out = np.zeros((7, n))
    filled = 0
    while filled < n:
        b = min(n - filled, 1 << 22)
        pos = x0 + rng.random((int(b * 1.1) + 16, 3)) * (xm - x0)
        pos = pos[np.sum((pos - c) ** 2, axis=1) > r * r][:b]
        k = pos.shape[0]
        out[0:3, filled:filled + k] = pos.T
        out[3:6, filled:filled + k] = rng.standard_normal((3, k)) * vth
        out[5, filled:filled + k] += V_DRIFT
        filled += k
    out[6] = cfg["mpw0"]
    return out


def make_world(E, cfg, form, P0, seed=11):
    """The sphere world with its initial state: P0 (host particles) or, when
    P0 is None, cfg["np"] ions loaded on the GPU by the drifting-Maxwellian
    loader (those inside the sphere are absorbed by the first push)."""
    ni, nj, nk = cfg["n"]
    w = E.World(ni, nj, nk, cfg["x0"], cfg["xm"])
    w.set_seed(seed)
    w.setTime(cfg["dt"], 1 << 30)
    w.addSphere(cfg["center"], cfg["radius"], cfg["phi_s"])
    w.addInlet()
    npart = cfg["np"] if P0 is None else P0.shape[1]
    cap = int(npart * 1.05) + (1 << 20)
    s = E.Species(w, "O+", 16 * AMU, QE, mpw0=cfg["mpw0"], capacity=cap, form=form,
                  walls=E.WALLS_ABSORB)
    src = E.BeamSource(s, V_DRIFT, N0, TI_EV * QE / K)
    sol = E.PotentialSolver(w, E.SOLVER_PCG, 1000, 1e-4)
    sol.setReferenceValues(PHI0, TE, N0)
    sol.setNewton(nr_max=20, nr_tol=NR_TOL, pcg_max=20000, pcg_tol=PCG_TOL,
                  fp32_inner=(form == E.FORM_MIXED))
    if P0 is None:
        s.loadParticlesBoxThermal(cfg["x0"], cfg["xm"], 0.0, npart, (0.0, 0.0, V_DRIFT), TI_EV * QE / K)
    else:
        s.set_particles(P0)
    if form == E.FORM_MIXED:
        s.sort()
    s.computeNumberDensity()
    w.computeChargeDensity()
    sol.solve()
    sol.computeEF()
    return w, s, src, sol


def timed_steps(E, torch, w, cfg, steps, warmup, flush):
    stream = torch.cuda.ExternalStream(w.stream_handle())
    for _ in range(warmup):
        w.step(cfg["sort_every"])
    w.sync()
    n_before = w.diag_row()[0]
    l0 = w.launches()
    s0 = w.solver_totals()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    torch.cuda.synchronize()
    for i in range(steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[i][0].record(stream)
        w.step(cfg["sort_every"])
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    w.sync()
    ms = [a.elapsed_time(b) for a, b in ev]
    n_after = w.diag_row()[0]
    l1 = w.launches()
    s1 = w.solver_totals()
    return dict(ms=ms, n=(n_before + n_after) / 2.0, launches=l1 - l0,
                solves=s1[0] - s0[0], newton=s1[1] - s0[1], inner=s1[2] - s0[2])


def deposit_alone(E, torch, w, s, reps=3):
    """The deposit outside the fused push: espic_deposit on the current ions
    (the accumulator cleared, k_deposit_mixed, k_density), CUDA events on the
    library's stream, after one untimed call.  The ions do not move, so the
    density it leaves is the one the step's fused deposit left."""
    stream = torch.cuda.ExternalStream(w.stream_handle())
    s.computeNumberDensity()
    w.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(reps)]
    for a, b in ev:
        with torch.cuda.stream(stream):
            a.record(stream)
        s.computeNumberDensity()
        with torch.cuda.stream(stream):
            b.record(stream)
    torch.cuda.synchronize()
    w.sync()
    return float(np.mean([a.elapsed_time(b) for a, b in ev]))


def profiled_steps(E, w, cfg, steps):
    w.profile(True)
    for _ in range(steps):
        w.step(cfg["sort_every"])
    ph, _ = w.profile_read()
    w.profile(False)
    return {k: v[0] / steps for k, v in ph.items()}, {k: v[1] / steps for k, v in ph.items()}


def e2e_steps(E, torch, w, s, src, sol, cfg, steps):
    """The Main-loop body through the C-ABI: injection uniforms H2D from pinned
    memory, the phases, the diag row D2H every step.  The uniforms of at most
    four steps are drawn (a 256x256x512 step takes 91 MB of them) and reused
    in turn: every step still copies its whole set from host memory."""
    import ctypes as C
    lib = E.lib()
    rng = np.random.default_rng(5)
    Lx = w.dh[0] * (w.ni - 1)
    Ly = w.dh[1] * (w.nj - 1)
    per = N0 * V_DRIFT * Lx * Ly * cfg["dt"] / cfg["mpw0"]
    nu = 1 + 13 * (int(per) + 2)
    slots = min(steps, 4)
    pinned = torch.empty((slots, nu), dtype=torch.float64, pin_memory=True)
    pinned.copy_(torch.from_numpy(rng.random((slots, nu))))
    row = torch.empty(7, dtype=torch.float64, pin_memory=True)
    used = E.I64()
    h2d = 0
    w.sync()
    t0 = time.perf_counter()
    for i in range(steps):
        ptr = C.cast(pinned[i % slots].data_ptr(), E.PD)
        E.check(lib.espic_source_sample_uniforms(w.h, src.id, ptr, nu, C.byref(used)))
        h2d += used.value * 8
        if cfg["sort_every"] and i % cfg["sort_every"] == 0:
            s.sort()
        s.advance(deposit=True)
        w.computeChargeDensity()
        sol.solve(wait=False)
        sol.computeEF()
        E.check(lib.espic_diag_row(w.h, C.cast(row.data_ptr(), E.PD), 7))
    el = time.perf_counter() - t0
    return dict(seconds=el, h2d=h2d / steps, d2h=7 * 8, n=float(row[0]))


def phi_error(E, w, cfg):
    """phi of the chosen (FP32-inner) solve against a tight FP64 Newton-PCG
    on the same charge density (the GPU's float64 solver, which the parity
    tests pin to the oracle's)."""
    phi_mixed = w.phi.copy()
    sol = E.PotentialSolver(w, E.SOLVER_PCG, 1000, 1e-4)
    sol.setReferenceValues(PHI0, TE, N0)
    sol.setNewton(nr_max=50, nr_tol=1e-11, pcg_max=40000, pcg_tol=1e-12, fp32_inner=False)
    conv, _, _, _ = sol.solve()
    phi64 = w.phi
    return float(np.max(np.abs(phi_mixed - phi64)) / np.max(np.abs(phi64))), bool(conv), phi64


def _err(a, b):
    d = np.asarray(a, dtype=np.float64) - np.asarray(b, dtype=np.float64)
    ref = np.abs(np.asarray(b, dtype=np.float64))
    return {"max_rel": float(np.max(np.abs(d)) / max(np.max(ref), 1e-300)),
            "rms_rel": float(np.sqrt(np.mean(d * d)) / max(np.sqrt(np.mean(ref * ref)), 1e-300))}


def oracle_errors(E, w, s, cfg, full, snap, phi64, conv64):
    """Errors of the chosen (mixed) form against the float64 oracle
    (oracle/espic_oracle.c) on the state of the last timed step:

    * ion density: the GPU's mixed deposit against the oracle's float64
      deposit (Field_::scatter, ch2/Field.h:164-183) of the same particles,
      widened exactly to float64 -- on every node (full) or on the node planes
      of a 33-plane slab through the sphere (cells outside the slab's
      particles do not touch it);
    * phi: the GPU's FP32-inner Newton-PCG result against the oracle's float64
      Newton-PCG on the oracle's charge density (full), or against the GPU's
      float64 Newton-PCG on the same density (phi64; the grid is too large
      for the host solve);
    * E: the GPU's computeEF of the mixed phi against the oracle's computeEF
      (ch2/PotentialSolver.cpp:70-110) of the float64 phi."""
    from oracle import pyoracle as po
    g = po.grid(cfg["n"], cfg["x0"], cfg["xm"])
    vol = w.read(E.FIELD_NODE_VOL)
    den_gpu, phi_gpu, ef_gpu = snap["den"], snap["phi"], snap["ef"]
    obj = w.object_id
    cell, off, vel = s.get_mixed()
    ni, nj, nk = cfg["n"]
    plane = ni * nj
    if full:
        sel = slice(None)
        k0, k1 = 0, nk - 1
    else:
        kc = int(round((cfg["center"][2] - cfg["x0"][2]) / ((cfg["xm"][2] - cfg["x0"][2]) / (nk - 1))))
        k0, k1 = kc - 16, kc + 16
        kk = cell >> 20
        sel = (kk >= k0 - 1) & (kk <= k1)
    P64 = po.from_mixed(g, np.ascontiguousarray(cell[sel]), np.ascontiguousarray(off[:, sel]),
                        np.ascontiguousarray(vel[:, sel]), cfg["mpw0"])
    del cell, off, vel
    den_o = po.divide_volume(po.deposit_fp64(g, P64), vol)
    del P64
    nodes = slice(k0 * plane, (k1 + 1) * plane)
    out = {"den": _err(den_gpu[nodes], den_o[nodes]), "den_nodes": "all" if full else "planes %d-%d" % (k0, k1)}
    if full:
        phi_o, conv, _, _ = po.newton_pcg(g, phi_gpu, den_o * QE, obj, PHI0, TE, N0, nr_max=50, nr_tol=1e-11,
                                          pcg_max=200000, pcg_tol=1e-12)
        out["phi_reference"] = "oracle float64 Newton-PCG on the oracle's density (converged: %s)" % conv
    else:
        phi_o = phi64
        out["phi_reference"] = "GPU float64 Newton-PCG on the same density (converged: %s)" % conv64
    out["phi"] = _err(phi_gpu, phi_o)
    ef_o = po.efield(g, phi_o)
    out["E"] = _err(ef_gpu, ef_o)
    out["E_reference"] = "oracle computeEF of that float64 phi"
    return out


def gpu_reference_algorithm_iterations(E, w, s, src, cfg):
    """Newton and PCG iterations of the reference's algorithm (Newton with a
    Jacobi-preconditioned CG in float64, no predictor) for one step of this
    state, on the GPU: the count the host baseline's per-iteration cost is
    multiplied by."""
    src.sample()
    s.advance(deposit=True)
    w.computeChargeDensity()
    sol = E.PotentialSolver(w, E.SOLVER_PCG, 1000, 1e-4)
    sol.setReferenceValues(PHI0, TE, N0)
    sol.setNewton(nr_max=20, nr_tol=NR_TOL, pcg_max=200000, pcg_tol=PCG_TOL, fp32_inner=False)
    sol.setMultigrid(0)
    sol.setPredictor(False)
    conv, nr, inner, _ = sol.solve()
    sol.setMultigrid(12)
    sol.setPredictor(True)
    return dict(newton=nr, pcg=inner, converged=bool(conv))


def _oracle_sphere(cfg):
    from oracle import pyoracle as po
    g = po.grid(cfg["n"], cfg["x0"], cfg["xm"])
    obj, phi = po.objects(g, cfg["center"], cfg["radius"], cfg["phi_s"])
    sph = np.array(list(cfg["center"]) + [cfg["radius"] ** 2])
    return po, g, obj, phi, sph


def cpu_sphere_steps(cfg, P0, threads, steps, warmup, seed=7):
    """The sphere step of ch3/ver2/Main.cpp:50-80 on this host's cores with
    the oracle port: warm-beam injection (ch4/Source.cpp:31-55), push with
    absorption and removal, fixed-point deposit (threaded over particle
    ranges like ch9/MT/Species.cpp:37-110), charge density, the serial
    Newton-PCG (Jacobi preconditioner, ch3/ver2/PotentialSolver.cpp:225-331,
    in its symmetric form, with the GPU path's inner stop rule) from the
    previous step's potential to the GPU arm's tolerances, and computeEF.  An initial cold solve precedes the
    steps, as in Main.cpp.  Every step is timed whole; returns the mean
    seconds per step, the mean particle count and the measured iterations."""
    import ctypes as C
    po, g, obj, phi, sph = _oracle_sphere(cfg)
    vol = po.node_volumes(g)
    M = 16 * AMU
    n = P0.shape[1]
    cap = n + 200_000
    P = np.zeros((7, cap))
    P[:, :n] = P0
    fx = 2.0 ** po.fixed_scale_exponent(cfg["mpw0"], cap)
    acc = np.zeros(g.nn, dtype=np.int64)
    nout = C.c_int64(0)
    L = po.lib()
    rng = np.random.default_rng(seed)

    def density(P, n):
        acc[:] = po.deposit_fixed(g, np.ascontiguousarray(P[:, :n]), fx)
        return po.density_from_fixed(acc, fx, vol)

    t0 = time.perf_counter()
    phi, conv0, nr0, pcg0, _ = po.newton_pcg_fallback(g, phi, density(P, n) * QE, obj, PHI0, TE, N0, 50, NR_TOL,
                                                      200000, PCG_TOL, 0, 0.0, early_stop=True)
    t_cold = time.perf_counter() - t0
    ef = po.efield(g, phi)
    times, counts, nrs, pcgs = [], [], [], []
    for st in range(warmup + steps):
        t0 = time.perf_counter()
        # inject (the GPU arm's beam source: ch4 warm beam)
        u = rng.random(1 + 13 * (int(N0 * V_DRIFT * 0.2 * 0.2 * cfg["dt"] / cfg["mpw0"]) + 2))
        used = C.c_int64(0)
        n = L.eo_inject_warm(C.byref(g), po.pd(ef), QE, M, cfg["dt"], cfg["mpw0"], V_DRIFT, N0, TI_EV * QE / K,
                             po.pd(u), C.byref(used), po.pd(P), cap, n, cap)
        assert n >= 0
        # push + removal + deposit, threaded
        L.eo_bench_push_deposit(C.byref(g), po.pd(ef), po.pd(sph), QE, M, cfg["dt"], fx, po.pd(P), cap, n, threads, 1,
                                C.byref(nout), po.pi64(acc))
        n = nout.value
        rho = po.density_from_fixed(acc, fx, vol) * QE
        phi, conv, nr, pcg, _ = po.newton_pcg_fallback(g, phi, rho, obj, PHI0, TE, N0, 20, NR_TOL, 200000, PCG_TOL,
                                                       0, 0.0, early_stop=True)
        ef = po.efield(g, phi)
        el = time.perf_counter() - t0
        if st >= warmup:
            times.append(el)
            counts.append(n)
            nrs.append(nr)
            pcgs.append(pcg)
    return dict(seconds=float(np.mean(times)), n=float(np.mean(counts)), newton=float(np.mean(nrs)),
                pcg=float(np.mean(pcgs)), cold_solve_s=t_cold, cold_pcg=pcg0, converged=bool(conv0))


def cpu_sample_costs(cfg, n_sample, threads, seed=1):
    """Per-particle cost of the threaded push + removal + deposit over a
    contiguous sample of the synthetic state, and the serial Newton-PCG's
    costs on the full grid: one residual evaluation (Newton iteration) and
    one Jacobi-PCG iteration, separated by timing runs of 1 and 3 PCG
    iterations."""
    import ctypes as C
    po, g, obj, phi, sph = _oracle_sphere(cfg)
    P = np.ascontiguousarray(synthetic_state(cfg, n_sample, seed))
    n = P.shape[1]
    fx = 2.0 ** po.fixed_scale_exponent(cfg["mpw0"], n)
    acc = np.zeros(g.nn, dtype=np.int64)
    nout = C.c_int64(0)
    ef = po.efield(g, phi)
    t_pd = po.lib().eo_bench_push_deposit(C.byref(g), po.pd(ef), po.pd(sph), QE, 16 * AMU, cfg["dt"], fx, po.pd(P),
                                          n, n, threads, 1, C.byref(nout), po.pi64(acc))
    rho = po.density_from_fixed(acc, fx, po.node_volumes(g)) * QE
    t = {}
    for it in (1, 3):
        t0 = time.perf_counter()
        po.newton_pcg(g, phi, rho, obj, PHI0, TE, N0, nr_max=1, nr_tol=0.0, pcg_max=it, pcg_tol=0.0)
        t[it] = time.perf_counter() - t0
    per_iter = (t[3] - t[1]) / 2
    return dict(pd_per_particle=t_pd / n, survive=nout.value / n, pcg_iter_s=per_iter,
                newton_res_s=max(t[1] - per_iter, 0.0), sample=n)


def c2_jacobi_iterations(threads, steps=3, warmup=1):
    """Newton and Jacobi-PCG iterations per step of the oracle's serial solve
    on the 64x64x128 sphere, measured on this host (cold solve, then steps
    warm-started from the previous potential)."""
    cfg = CONFIGS["sphere64"]
    r = cpu_sphere_steps(cfg, synthetic_state(cfg, cfg["np"], 1), threads, steps, warmup)
    return r


def run_reference(args):
    if args.config == "dsmc41":
        run_reference_dsmc(args)
        return
    if not args.config.startswith("sphere"):
        print(json.dumps({"impl": "reference", "unavailable": "the reference arm times the sphere workloads "
                          "(the workload the metric is quoted on); run it with --config sphere64 or sphere256"}))
        return
    cfg = CONFIGS[args.config]
    threads = os.cpu_count() or 1
    if args.config == "sphere64":
        # every step measured whole, on the GPU arm's initial state and ion count
        P0 = synthetic_state(cfg, cfg["np"], 1)
        # a host step takes seconds: at most 6 timed steps after 1 warm-up
        ksteps, kwarm = min(args.steps, 6), min(args.warmup, 1)
        r = cpu_sphere_steps(cfg, P0, threads, ksteps, kwarm)
        v = r["n"] / r["seconds"]
        sample = ("%d whole steps after %d warm-up steps (inject, threaded push+removal+deposit on %d threads, "
                  "serial Newton-PCG with Jacobi preconditioner from the previous potential: %.2f Newton and %.1f "
                  "PCG iterations per step measured, computeEF) over %.0f ions; cold initial solve %.1f s "
                  "(%d PCG iterations)" % (ksteps, kwarm, threads, r["newton"], r["pcg"], r["n"],
                                            r["cold_solve_s"], r["cold_pcg"]))
        extra = {"newton_per_step": r["newton"], "pcg_iterations_per_step": r["pcg"],
                 "poisson_ms_per_step": None}
        ms = 1e3 * r["seconds"]
        particles = r["n"]
    else:
        # the 256x256x512 case cannot run whole on the host (a single step's
        # serial solve takes minutes): a bounded sample, stated
        c2 = c2_jacobi_iterations(threads)
        c2cfg = CONFIGS["sphere64"]
        refine = max((c2cfg["xm"][d] - c2cfg["x0"][d]) / (c2cfg["n"][d] - 1) /
                     ((cfg["xm"][d] - cfg["x0"][d]) / (cfg["n"][d] - 1)) for d in range(3))
        vals = []
        for i in range(args.warmup + args.steps):
            c = cpu_sample_costs(cfg, 20_000_000, threads, seed=1 + i)
            if i >= args.warmup:
                vals.append(c)
        pd_pp = float(np.mean([c["pd_per_particle"] for c in vals]))
        it_s = float(np.mean([c["pcg_iter_s"] for c in vals]))
        res_s = float(np.mean([c["newton_res_s"] for c in vals]))
        particles = cfg["np"] * float(np.mean([c["survive"] for c in vals]))
        pcg = c2["pcg"] * refine
        solve_s = c2["newton"] * res_s + pcg * it_s
        step_s = particles * pd_pp + solve_s
        v = particles / step_s
        ms = 1e3 * step_s
        sample = ("per step: threaded push+removal+deposit of a 20M-ion sample (%d threads) scaled to %.0f ions; "
                  "serial Newton-PCG costs on the full grid (residual %.3f s, Jacobi-PCG iteration %.3f s, "
                  "measured) x the iterations per step measured on this host at 64x64x128 (%.2f Newton, %.1f PCG, "
                  "warm-started steps after a cold solve) with the PCG count scaled by the grid refinement %.2f "
                  "(Jacobi-PCG iterations grow as 1/h): %.0f PCG iterations per step"
                  % (threads, particles, res_s, it_s, c2["newton"], c2["pcg"], refine, pcg))
        extra = {"newton_per_step": c2["newton"], "pcg_iterations_per_step": pcg,
                 "poisson_ms_per_step": 1e3 * solve_s, "c2_measured": {"newton": c2["newton"], "pcg": c2["pcg"]}}
    line = {"metric": METRIC, "value": v, "unit": "particle-steps/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.config, "grid": list(cfg["n"]), "particles": particles},
            "cpu_baseline": {"value": v, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    line.update(extra)
    print(json.dumps(line))


def ncu_case(args):
    """The workload's state, then exactly one push with the fused deposit
    (k_push_tiles after the tile sort) and one k_newton_pcg<float> launch:
    the case profiled with ncu -k regex:"k_push_tiles|k_newton_pcg" -c 2."""
    E = espic_module()
    if not os.path.exists(E.LIB_PATH):
        E.build()
    if args.config == "ensemble512":
        cfg = dict(CONFIGS["ensemble512"])
        cfg["nbox"] = args.ncu_boxes or cfg["nbox"]
        ens, npart, _ = make_ensemble(E, cfg)
        ens.set_launch(4096, 512, 1024)
        ens.step(1, graph=False)
        sweeps, conv, _ = ens.status()
        print(json.dumps({"ncu_case": "ensemble", "boxes": cfg["nbox"], "particles": npart,
                          "sweeps_mean": float(sweeps.mean()), "converged": int(conv.sum())}))
        ens.close()
        return
    cfg = CONFIGS[args.config]
    npart = args.ncu_particles or cfg["np"]
    ni, nj, nk = cfg["n"]
    w = E.World(ni, nj, nk, cfg["x0"], cfg["xm"])
    w.setTime(cfg["dt"], 100)
    w.addSphere(cfg["center"], cfg["radius"], cfg["phi_s"])
    w.addInlet()
    s = E.Species(w, "O+", 16 * AMU, QE, mpw0=cfg["mpw0"] * cfg["np"] / npart, capacity=int(npart * 1.5),
                  form=E.FORM_MIXED, walls=E.WALLS_ABSORB)
    sol = E.PotentialSolver(w, E.SOLVER_PCG, 1000, 1e-4)
    sol.setReferenceValues(PHI0, TE, N0)
    sol.setNewton(nr_max=20, nr_tol=NR_TOL, pcg_max=20000, pcg_tol=PCG_TOL, fp32_inner=True)
    s.loadParticlesBoxThermal(cfg["x0"], cfg["xm"], 0.0, npart, (0.0, 0.0, V_DRIFT), TI_EV * QE / K)
    s.sort()
    sol.computeEF()
    s.advance(deposit=True)
    w.computeChargeDensity()
    print(json.dumps({"ncu_case": args.config, "solve": sol.solve(), "particles": s.getNp()}))
    w.close()


def aggregate(ms_step, n_local, dist, device):
    """Max step time over ranks and the whole-job throughput (units all ranks
    processed / that time), as the replica runs of --gpus N report it."""
    import torch
    world_size = dist.get_world_size() if dist else 1
    if dist:
        t = torch.tensor([ms_step, n_local], dtype=torch.float64, device=device)
        tmax = t.clone()
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        tsum = t.clone()
        dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
        return float(tmax[0]), float(tsum[1]) / (float(tmax[0]) * 1e-3), world_size
    return ms_step, n_local / (ms_step * 1e-3), 1


def run_box(args, E, torch, dist, rank, world_size):
    """Configuration 1: the ch2 grounded box, 80,000 O+ uniform at n = 1e11
    and 10,000 electrons in the octant [-0.1,0]^2 x [0,0.1], zero velocity,
    dt = 2e-10, red-black SOR (omega 1.4) to L2 residual 1e-4; FP64 plain
    form (bit-exact with the reference's arithmetic)."""
    cfg = CONFIGS["box21"]
    QE_, AMU_, ME_ = E.QE, E.AMU, E.ME

    def world():
        w = E.World(*cfg["n"], cfg["x0"], cfg["xm"])
        w.set_seed(1 + rank)
        w.setTime(cfg["dt"], 1 << 30)
        si = E.Species(w, "O+", 16 * AMU_, QE_, capacity=1 << 17)
        se = E.Species(w, "e-", ME_, -QE_, capacity=1 << 15)
        si.loadParticlesBox(cfg["x0"], cfg["xm"], 1e11, 80000)
        se.loadParticlesBox(cfg["x0"], (0.0, 0.0, 0.1), 1e11, 10000)
        sol = E.PotentialSolver(w, E.SOLVER_SOR, 10000, 1e-4)
        sol.solve()
        sol.computeEF()
        return w
    w = world()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    if dist:
        dist.barrier()
    clocks = Clocks()
    clocks.start()
    t = timed_steps(E, torch, w, cfg, args.steps, args.warmup, flush)
    ck = clocks.stop()
    ms = float(np.sum(t["ms"])) / args.steps
    ms_max, value, ws = aggregate(ms, 90000.0, dist, "cuda")
    phases, _ = profiled_steps(E, w, cfg, max(3, min(args.steps, 10)))
    w.close()
    # e2e: the ch2 loop body through the C-ABI, diag row read back each step
    w = world()
    for _ in range(args.warmup):
        w.step(0)
    row = np.zeros(13)
    w.sync()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        w.step(0, row)
    e2e_s = (time.perf_counter() - t0) / args.steps
    w.close()
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "box21", "grid": list(cfg["n"]), "particles": 90000, "form": "fp64 plain",
                       "solver": "red-black SOR, omega 1.4, tol 1e-4",
                       "l2": "flushed between timed steps (256 MB write, outside the events)"},
            "poisson_ms_per_step": phases["solve"], "phase_ms_per_step": phases,
            "sor_iterations_per_step": t["newton"] / args.steps,
            "e2e": {"value": 90000.0 * ws / e2e_s, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 13 * 8},
            "gpu_launches": t["launches"], "clocks": ck}
    if rank == 0:
        print(json.dumps(line))


def ensemble_spec(cfg):
    """Per box: nodes per axis uniform in 16..64, macroparticles log-uniform
    in [1e4, 2e6] (half O+, half e-), density log-uniform in [1e10, 1e12],
    the electron octant drawn from the 8 octants of the box."""
    rng = np.random.default_rng(cfg["seed"])
    nb = cfg["nbox"]
    nodes = rng.integers(16, 65, size=(nb, 3))
    npart = np.exp(rng.uniform(np.log(1e4), np.log(2e6), size=nb)).astype(np.int64)
    dens = np.exp(rng.uniform(np.log(1e10), np.log(1e12), size=nb))
    octant = rng.integers(0, 8, size=nb)
    n_i = npart // 2
    n_e = npart - n_i
    x0, xm = np.array(cfg["x0"]), np.array(cfg["xm"])
    V = np.prod(xm - x0)
    mpw = np.stack([dens * V / n_i, dens * V / 8 / n_e], axis=1)
    return nodes, n_i, n_e, octant, mpw


def make_ensemble(E, cfg, boxes=None):
    """The ensemble of cfg's boxes, or of the subset `boxes` (their ids in
    the whole ensemble key their random streams, so each box loads the same
    particles whichever rank owns it)."""
    nodes, n_i, n_e, octant, mpw = ensemble_spec(cfg)
    ids = np.arange(cfg["nbox"]) if boxes is None else np.asarray(boxes, dtype=np.int64)
    x0, xm = np.array(cfg["x0"]), np.array(cfg["xm"])
    ens = E.Ensemble(nodes[ids], x0, xm, [16 * AMU, E.ME], [QE, -QE], mpw[ids],
                     np.stack([n_i[ids], n_e[ids]], axis=1), cfg["dt"])
    if boxes is not None:
        ens.set_box_ids(ids)
    mid = (x0 + xm) / 2
    for local, b in enumerate(ids):
        ens.load_box(local, 0, x0, xm, n_i[b])
        lo = np.where((octant[b] >> np.arange(3)) & 1, mid, x0)
        hi = np.where((octant[b] >> np.arange(3)) & 1, xm, mid)
        ens.load_box(local, 1, lo, hi, n_e[b])
    ens.set_solver(10000, 1e-4, 0.0)
    ens.prepare()
    return ens, int(n_i[ids].sum() + n_e[ids].sum()), nodes[ids]


def ensemble_shard(E, cfg, rank, world_size):
    """The boxes this rank steps: the whole ensemble split by work
    (particles + nodes) with no exchange between ranks."""
    if world_size <= 1:
        return None
    nodes, n_i, n_e, _, _ = ensemble_spec(cfg)
    owner, _ = E.partition_boxes(E.ensemble_work(nodes, n_i + n_e), world_size)
    return np.nonzero(owner == rank)[0]


def ensemble_cpu_baseline(E, ens, nodes, cfg, nsample=3):
    """The oracle on a sample of boxes, one thread: push + fixed-point deposit
    of both species and the red-black SOR (omega 1.4) from the GPU's
    potential to the same tolerance."""
    from oracle import pyoracle as po
    order = np.argsort(np.prod(nodes, axis=1))
    pick = order[np.linspace(0, len(order) - 1, nsample).astype(int)]
    tot_p, tot_s = 0, 0.0
    for b in pick:
        g = po.grid(nodes[b], cfg["x0"], cfg["xm"])
        phi = ens.read(int(b), E.FIELD_PHI)
        ef = po.efield(g, phi)
        vol = po.node_volumes(g)
        dens = []
        t0 = time.perf_counter()
        for sp, (q, m) in enumerate(((QE, 16 * AMU), (-QE, E.ME))):
            P = ens.particles(int(b), sp)
            fx = 2.0 ** po.fixed_scale_exponent(float(P[6, 0]), P.shape[1])
            P = po.push_box(g, ef, q, m, cfg["dt"], P)
            dens.append(po.density_from_fixed(po.deposit_fixed(g, P, fx), fx, vol))
            tot_p += P.shape[1]
        rho = po.charge_density([QE, -QE], np.stack(dens))
        po.sor_box(g, phi, rho, 10000, 1e-4, "rb")
        tot_s += time.perf_counter() - t0
    return dict(value=tot_p / tot_s, unit="particle-steps/s", cores=1, kind="port",
                sample="one step (push, deposit, red-black SOR omega 1.4 from the GPU potential) of %d boxes "
                       "with %d particles, single thread" % (nsample, tot_p))


def run_ensemble(args, E, torch, dist, rank, world_size):
    """The batched ensemble: 512 ch2 boxes in one step graph (push + deposit
    over a work list, per-box SOR + E), FP32 particles under an FP64
    residual, tol 1e-4, the per-box optimal red-black factor."""
    cfg = CONFIGS["ensemble512"]
    mine = ensemble_shard(E, cfg, rank, world_size)
    ens, npart, nodes = make_ensemble(E, cfg, mine)
    tune = ens.autotune()
    stream = torch.cuda.ExternalStream(ens.stream_handle())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ens.step(args.warmup)
    ens.sync()
    l0 = ens.launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks()
    clocks.start()
    torch.cuda.synchronize()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[i][0].record(stream)
        ens.step(1)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ens.sync()
    launches = ens.launches() - l0
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    sweeps, conv, res = ens.status()
    ms_max, value, ws = aggregate(ms, float(npart), dist, "cuda")
    # e2e: the public step call plus the per-box solve status read back
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ens.step(1)
        ens.status()
    e2e_s = (time.perf_counter() - t0) / args.steps
    _, e2e_value, _ = aggregate(1e3 * e2e_s, float(npart), dist, "cuda")
    hbm, kind = peaks()
    push_gbs = 56.0 * npart / (tune["push_ms"] * 1e-3) / 1e9
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max, "higher_is_better": True, "scaling": "strong",
            "vs_baseline": None, "dtype": "f32+i32 particles, f32 SOR sweeps under f64 residual",
            "data": "synthetic",
            "config": {"workload": "ensemble512", "boxes": cfg["nbox"], "boxes_rank0": int(len(nodes)),
                       "particles_rank0": npart, "parallelism": "boxes split by work over %d ranks" % ws,
                       "nodes": int(np.prod(nodes, axis=1).sum()), "solver": "red-black SOR, per-box optimal "
                       "omega, tol 1e-4", "launch": {k: tune[k] for k in ("chunk", "push_threads",
                                                                        "solve_threads", "cluster")},
                       "l2": "flushed between timed steps (256 MB write, outside the events)"},
            "phase_ms_per_step": {"push": tune["push_ms"], "solve": tune["solve_ms"]},
            "sor_sweeps_per_step": {"mean": float(np.mean(sweeps)), "max": int(np.max(sweeps))},
            "converged_boxes": int(conv.sum()),
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": int(len(nodes) * 16)},
            "gpu_launches": launches,
            "roofline_push": {"bound": "hbm", "kernel": "k_ens_push", "achieved": push_gbs, "peak": hbm,
                              "unit": "GB/s", "frac": push_gbs / hbm, "bytes_per_particle": 56,
                              "peak_kind": kind},
            "clocks": ck}
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = ensemble_cpu_baseline(E, ens, nodes, cfg)
    ens.close()
    if rank == 0:
        print(json.dumps(line))


def run_diff(args, E, torch):
    """The differentiable sphere run: 500k O+ (drifting Maxwellian, 7 km/s,
    0.1 eV) in the 32x32x64 sphere box, 400 steps, loss = normalised final
    field energy + normalised wake-box ion count, gradients with respect to the
    sphere potential, the drift velocity and the initial state by the adjoint
    kernels (checkpoints every 20 steps), checked by central differences and
    against the FP32 adjoint.  The unit is particle-steps/s of one forward +
    backward pass."""
    cfg = CONFIGS["diff32"]
    n, steps = cfg["np"], cfg["steps"]
    rng = np.random.default_rng(11)
    x0, xm = np.array(cfg["x0"]), np.array(cfg["xm"])
    c = np.array(cfg["center"])
    pos = x0 + rng.random((3 * n, 3)) * (xm - x0)
    pos = pos[np.sum((pos - c) ** 2, axis=1) > (cfg["radius"] + 0.005) ** 2][:n]
    X = np.ascontiguousarray(pos.T)
    vth = rng.normal(0, np.sqrt(TI_EV * QE / (16 * AMU)), (3, n))
    dh = np.min((xm - x0) / (np.array(cfg["n"]) - 1))
    V = np.prod(xm - x0) - 4.0 / 3.0 * np.pi * cfg["radius"] ** 3

    def world(fp32):
        w = E.World(*cfg["n"], cfg["x0"], cfg["xm"])
        w.setTime(cfg["dt"], 1 << 30)
        w.addSphere(cfg["center"], cfg["radius"], cfg["phi_s"])
        w.addInlet()
        sol = E.PotentialSolver(w, E.SOLVER_PCG, 100, 1e-4)
        sol.setReferenceValues(PHI0, TE, N0)
        sol.setNewton(nr_max=60, nr_tol=1e-12, pcg_max=5000, pcg_tol=1e-10, fp32_inner=fp32)
        return w

    def vel(vd):
        v = vth.copy()
        v[2] += vd
        return v

    kw = dict(n=n, mass=16 * AMU, charge=QE, mpw0=N0 * V / n, delta=0.5 * dh, wake_z=cfg["wake"],
              checkpoint_every=cfg["checkpoint"])
    w = world(False)
    scale = []
    for a, b in ((1.0, 0.0), (0.0, 1.0)):
        with E.DiffRun(w, alpha=a, beta=b, **kw) as r:
            r.set_state(X, vel(V_DRIFT))
            scale.append(1.0 / r.forward(cfg["phi_s"], steps))
    out = {}
    for prec in ("fp64", "fp32"):
        wp = world(prec == "fp32")
        with E.DiffRun(wp, alpha=scale[0], beta=scale[1], precision=prec, **kw) as r:
            r.set_state(X, vel(V_DRIFT))
            r.forward(cfg["phi_s"], steps)
            r.backward()  # warm-up
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            L = r.forward(cfg["phi_s"], steps)
            t1 = time.perf_counter()
            g = r.backward()
            t2 = time.perf_counter()
            out[prec] = dict(L=L, g=g, fwd=t1 - t0, bwd=t2 - t1)
            if prec == "fp64":
                def loss(ps=cfg["phi_s"], v=None):
                    r.set_state(X, vel(V_DRIFT) if v is None else v)
                    return r.forward(ps, steps)
                out["fd"] = {}
                for h in (1e-3, 1e-5, 1e-7):
                    fd_ps = (loss(ps=cfg["phi_s"] * (1 + h)) - loss(ps=cfg["phi_s"] * (1 - h))) / (
                        2 * cfg["phi_s"] * h)
                    fd_vd = (loss(v=vel(V_DRIFT * (1 + h))) - loss(v=vel(V_DRIFT * (1 - h)))) / (2 * V_DRIFT * h)
                    out["fd"][h] = dict(phi_s=fd_ps, vd=fd_vd)
        wp.close()
    w.close()
    g64, g32 = out["fp64"]["g"], out["fp32"]["g"]
    t = out["fp64"]["fwd"] + out["fp64"]["bwd"]
    relerr = lambda a, b: abs(a - b) / abs(b)
    line = {"metric": METRIC, "value": n * steps / t, "unit": "particle-steps/s (forward + adjoint)",
            "n_gpus": 1, "steps": steps, "warmup": 1, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64 particles and adjoint (f32 form beside)",
            "data": "synthetic",
            "config": {"workload": "diff32", "grid": list(cfg["n"]), "particles": n, "steps": steps,
                       "checkpoint_every": cfg["checkpoint"], "absorber_layer_m": 0.5 * dh},
            "forward_s": out["fp64"]["fwd"], "backward_s": out["fp64"]["bwd"],
            "fp32": {"forward_s": out["fp32"]["fwd"], "backward_s": out["fp32"]["bwd"]},
            "gradients": {"dL_dphi_sphere": g64[0], "dL_dv_drift": float(g64[2][2].sum())},
            "fd_rel_err": {"h=%g" % h: {"phi_sphere": relerr(f["phi_s"], g64[0]),
                                        "v_drift": relerr(f["vd"], float(g64[2][2].sum()))}
                           for h, f in out["fd"].items()},
            "fd_note": "central differences converge to the adjoint as h -> 0; over 400 steps the loss is "
                       "linear only below ~1e-7 relative (perturbations grow through the particle dynamics), "
                       "so a 1e-3 step measures a secant",
            "fp32_vs_fp64_rel": {"phi_sphere": relerr(g32[0], g64[0]),
                                 "v_drift": relerr(float(g32[2][2].sum()), float(g64[2][2].sum()))}}
    print(json.dumps(line))


def run_dsmc(args, E, torch):
    """DSMC_MEX::apply (ch4/Collisions.cpp:108-183) over the ch4 neutral gas:
    6.4M O atoms in 32,000 cells (about 200 per cell) with the counter-based
    stream, timed with CUDA events on the library's stream; the L2 is
    flushed between timed calls.  The CPU baseline is the oracle's
    restatement of the same call on the same atoms (one thread)."""
    cfg = CONFIGS["dsmc41"]
    x0, xm = np.array(cfg["x0"]), np.array(cfg["xm"])
    n = int(round(cfg["nda"] * np.prod(xm - x0) / cfg["mpw0"]))
    mass, dt = 16 * AMU, cfg["dt"]
    w = E.World(*cfg["n"], cfg["x0"], cfg["xm"])
    w.set_seed(7)
    w.setTime(dt, 1 << 30)
    s = E.Species(w, "O", mass, 0.0, mpw0=cfg["mpw0"], capacity=n + 1024, form=E.FORM_FP64)
    s.loadParticlesBoxThermal(cfg["x0"], cfg["xm"], 0.0, n, (0.0, 0.0, V_DRIFT), cfg["temp"])
    s.enable_dsmc()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.ExternalStream(w.stream_handle())
    for _ in range(max(args.warmup, 3)):
        s.dsmc(dt)
    w.sync()
    _, _, tot0 = s.dsmc_status()
    l0 = w.launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = Clocks()
    clocks.start()
    torch.cuda.synchronize()
    for i in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
            ev[i][0].record(stream)
        s.dsmc(dt)
        with torch.cuda.stream(stream):
            ev[i][1].record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    ms = float(np.mean([a.elapsed_time(b) for a, b in ev]))
    launches = w.launches() - l0
    smax, _, tot1 = s.dsmc_status()
    # e2e: the call through the C-ABI plus the read of its status
    t0 = time.perf_counter()
    for _ in range(args.steps):
        s.dsmc(dt)
        s.dsmc_status()
    e2e_s = (time.perf_counter() - t0) / args.steps

    def timed(fn):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(args.steps)]
        fn()
        torch.cuda.synchronize()
        for i in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
                evs[i][0].record(stream)
            fn()
            with torch.cuda.stream(stream):
                evs[i][1].record(stream)
        torch.cuda.synchronize()
        return float(np.mean([a.elapsed_time(b) for a, b in evs]))

    # ch4 species moments (Species::sampleMoments) and MCC_CEX::apply with
    # the same atoms as source and target (den and stream velocity of the gas)
    ms_mom = timed(s.sampleMoments)
    s.computeGasProperties()
    s.computeNumberDensity()
    mcc = E.MCC_CEX(s, s, w)
    ms_mcc = timed(lambda: mcc.apply(dt))
    P = s.particles()
    # the ch4 neutral push (no sphere here: atoms leave through the faces)
    n_before = s.getNp()
    ms_push = timed(s.advance_ch4)
    n_after = s.getNp()
    w.close()
    # CPU: the oracle on the same atoms, starting from the warmed-up sigma_cr_max
    _, _, cpu_t = dsmc_cpu_calls(cfg, P, smax, 2)
    n_cells = (cfg["n"][0] - 1) * (cfg["n"][1] - 1) * (cfg["n"][2] - 1)
    hbm, peak_kind = peaks()
    alg = 40.0 * n
    achieved = alg / (ms * 1e-3) / 1e9
    line = {"metric": "DSMC_MEX particle-calls/s (ch4 neutral gas)", "value": n / (ms * 1e-3),
            "unit": "particle-calls/s", "n_gpus": 1, "steps": args.steps, "warmup": max(args.warmup, 3),
            "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": "dsmc41", "grid": list(cfg["n"]), "particles": n, "cells": n_cells,
                       "density": cfg["nda"], "temp_K": cfg["temp"], "mpw0": cfg["mpw0"], "dt": dt,
                       "l2": "flushed between timed calls (256 MB write, outside the events)"},
            "collisions_per_call": (tot1 - tot0) / args.steps, "sigma_cr_max": smax,
            "e2e": {"value": n / e2e_s, "unit": "particle-calls/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 24},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "kernel": "one DSMC call (k_dsmc_cells, scan, k_dsmc_scatter, "
                         "k_dsmc_collide)", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "traffic": None, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": alg, "bytes_per_particle": 40},
            "clocks": ck,
            "cpu_baseline": {"value": n / float(np.mean(cpu_t)), "unit": "particle-calls/s", "cores": 1,
                             "kind": "port", "sample": "2 calls of the oracle's DSMC_MEX over all %d atoms" % n},
            "sample_moments": {"ms_per_call": ms_mom, "particles_per_s": n / (ms_mom * 1e-3),
                               "bytes_per_particle": 56,
                               "hbm_frac": 56.0 * n / (ms_mom * 1e-3) / 1e9 / hbm},
            "mcc_cex": {"ms_per_call": ms_mcc, "particles_per_s": n / (ms_mcc * 1e-3), "bytes_per_particle": 48,
                        "hbm_frac": 48.0 * n / (ms_mcc * 1e-3) / 1e9 / hbm},
            "ch4_push": {"ms_per_call": ms_push, "particles": [n_before, n_after],
                         "particles_per_s": 0.5 * (n_before + n_after) / (ms_push * 1e-3), "bytes_per_particle": 96,
                         "hbm_frac": 96.0 * 0.5 * (n_before + n_after) / (ms_push * 1e-3) / 1e9 / hbm}}
    print(json.dumps(line))


def dsmc_cpu_calls(cfg, P, smax, calls, seed=3):
    """`calls` DSMC_MEX::apply calls of the oracle's restatement on the atoms P
    (one host thread), each with fresh uniforms drawn beforehand (room for
    sigma_cr_max to grow fourfold).  Returns (P, sigma_cr_max, seconds per
    call)."""
    from oracle import pyoracle as po
    x0, xm, n3 = np.array(cfg["x0"]), np.array(cfg["xm"]), np.array(cfg["n"])
    g = po.grid(cfg["n"], cfg["x0"], cfg["xm"])
    mass, dt, dh = 16 * AMU, cfg["dt"], (xm - x0) / (n3 - 1)
    ci, cj = cfg["n"][0] - 1, cfg["n"][1] - 1
    rng = np.random.default_rng(seed)
    times = []
    for _ in range(calls):
        ijk = ((P[0:3] - x0[:, None]) / dh[:, None]).astype(np.int64)
        cnt = np.bincount(ijk[2] * cj * ci + ijk[1] * ci + ijk[0], minlength=ci * cj * (cfg["n"][2] - 1))
        ng = np.floor(0.5 * cnt * cnt * cfg["mpw0"] * (4 * smax) * dt / np.prod(dh) + 0.5)
        u = rng.random(int(8 * ng.sum()) + 100_000)
        t0 = time.perf_counter()
        P, smax, _, used, _ = po.dsmc_mex(g, mass, cfg["mpw0"], dt, po_c(mass), smax, P, u)
        times.append(time.perf_counter() - t0)
        assert used <= u.size
    return P, smax, times


def dsmc_state(cfg, seed):
    """the dsmc41 gas on the host: atoms uniform in the box, drifting
    Maxwellian velocities (7 km/s along z, 1000 K), weight mpw0"""
    x0, xm = np.array(cfg["x0"]), np.array(cfg["xm"])
    n = int(round(cfg["nda"] * np.prod(xm - x0) / cfg["mpw0"]))
    rng = np.random.default_rng(seed)
    P = np.empty((7, n))
    P[0:3] = x0[:, None] + rng.random((3, n)) * (xm - x0)[:, None]
    P[3:6] = rng.standard_normal((3, n)) * np.sqrt(K * cfg["temp"] / (16 * AMU))
    P[5] += V_DRIFT
    P[6] = cfg["mpw0"]
    return P


def run_reference_dsmc(args):
    """--impl reference on dsmc41: the oracle's DSMC_MEX restatement on the
    host (the reference's own ch4 code is not on the GPU host), warm-up
    calls from the reference's starting sigma_cr_max, then timed calls."""
    cfg = CONFIGS["dsmc41"]
    P = dsmc_state(cfg, 7)
    n = P.shape[1]
    P, sm, _ = dsmc_cpu_calls(cfg, P, 1e-14, max(args.warmup, 0), seed=5)
    _, _, t = dsmc_cpu_calls(cfg, P, sm, args.steps, seed=6)
    v = n / float(np.mean(t))
    line = {"metric": "DSMC_MEX particle-calls/s (ch4 neutral gas)", "value": v, "unit": "particle-calls/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * float(np.mean(t)), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "dsmc41", "grid": list(cfg["n"]), "particles": n},
            "cpu_baseline": {"value": v, "unit": "particle-calls/s", "cores": 1, "kind": "port",
                             "sample": "%d timed calls of the oracle's DSMC_MEX over all %d atoms after %d warm-up "
                                       "calls" % (args.steps, n, args.warmup)},
            "e2e": {"value": v, "unit": "particle-calls/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def po_c(mass):
    """DSMC_MEX's VHS parameters for one species (ch4/Collisions.h:53-60)"""
    import math
    mr = mass * mass / (mass + mass)
    return np.array([4.07e-10, 0.77, 2 * K * 273.15 / mr, math.gamma(2.5 - 0.77)])


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="espic", choices=["espic", "reference"])
    ap.add_argument("--config", default="sphere256", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain form")
    ap.add_argument("--sort-every", type=int, default=0,
                    help="steps between counting sorts of the mixed particles (default: the workload's)")
    ap.add_argument("--ncu-case", action="store_true",
                    help="one push + one solve of the workload (mixed form), for an ncu capture")
    ap.add_argument("--ncu-particles", type=int, default=0,
                    help="ions of the --ncu-case state (default: the workload's); keeps captures small")
    ap.add_argument("--ncu-boxes", type=int, default=0,
                    help="boxes of the ensemble --ncu-case (default: the workload's)")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world_size = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    if args.ncu_case:
        ncu_case(args)
        return

    import torch
    dist = None
    if world_size > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    E = espic_module()
    if not os.path.exists(E.LIB_PATH):
        E.build()
    if args.config == "box21":
        run_box(args, E, torch, dist, rank, world_size)
        if dist:
            dist.destroy_process_group()
        return
    if args.config == "diff32":
        run_diff(args, E, torch)
        return
    if args.config == "dsmc41":
        run_dsmc(args, E, torch)
        return
    if args.config == "ensemble512":
        run_ensemble(args, E, torch, dist, rank, world_size)
        if dist:
            dist.destroy_process_group()
        return
    cfg = dict(CONFIGS[args.config])
    if args.sort_every:
        cfg["sort_every"] = args.sort_every
    big = cfg["np"] > 50_000_000
    # large cases are loaded on the GPU; the CPU baseline then uses a sample
    P0 = None if big else synthetic_state(cfg, cfg["np"], 1 + rank)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    # mixed form: the chosen form
    w, s, src, sol = make_world(E, cfg, E.FORM_MIXED, P0)
    if dist:
        dist.barrier()
    clocks = Clocks()
    clocks.start()
    t = timed_steps(E, torch, w, cfg, args.steps, args.warmup, flush)
    ck = clocks.stop()
    ms_step, value, _ = aggregate(float(np.sum(t["ms"])) / args.steps, t["n"], dist, "cuda")
    dep_ms = deposit_alone(E, torch, w, s)
    # one whole sort period, so the sort's share of a step is in the table
    phases, counts = profiled_steps(E, w, cfg, cfg["sort_every"] or max(3, min(args.steps, 10)))
    snap = {"den": s.den, "phi": w.phi.copy(), "ef": w.ef}
    err, conv64, phi64 = phi_error(E, w, cfg)
    errs = oracle_errors(E, w, s, cfg, not big, snap, phi64, conv64)
    ref_it = gpu_reference_algorithm_iterations(E, w, s, src, cfg)
    inner_per_step = t["inner"] / max(args.steps, 1)
    # e2e through the C-ABI (a fresh world, same state)
    w.close()
    w, s, src, sol = make_world(E, cfg, E.FORM_MIXED, P0)
    for _ in range(args.warmup):
        w.step(cfg["sort_every"])
    # one whole sort period, as the timed steps amortise the sort
    e2e_n = (cfg["sort_every"] or args.steps) if big else args.steps
    e = e2e_steps(E, torch, w, s, src, sol, cfg, e2e_n)
    w.close()

    # plain FP64 form
    fp64 = None
    if not args.no_fp64:
        w, s, src, sol = make_world(E, cfg, E.FORM_FP64, P0)
        k64 = max(3, args.steps // 4)
        t64 = timed_steps(E, torch, w, cfg, k64, 2, flush)
        ph64, _ = profiled_steps(E, w, cfg, 3)
        ms64 = float(np.sum(t64["ms"])) / k64
        fp64 = {"value": t64["n"] / (ms64 * 1e-3), "ms_per_step": ms64, "poisson_ms_per_step": ph64["solve"],
                "push_ms": ph64["push"], "steps": k64}
        w.close()

    # roofline of the dominant kernel and of the push
    hbm, peak_kind = peaks()
    ni, nj, nk = cfg["n"]
    n_unknown = (ni - 2) * (nj - 2) * (nk - 2)
    dom = max(phases, key=lambda k: phases[k])
    # after a sort the push runs one block per tile segment (k_push_tiles);
    # grids narrower than a tile box keep the per-particle k_push_mixed
    push_kernel = "k_push_tiles" if min(cfg["n"]) >= 13 and cfg["sort_every"] else "k_push_mixed"
    push_bytes = 56.0 * t["n"]
    push_gbs = push_bytes / (phases["push"] * 1e-3) / 1e9
    if dom == "solve":
        alg = 24.0 * n_unknown * inner_per_step
        achieved = alg / (phases["solve"] * 1e-3) / 1e9
        kname = "k_newton_pcg<float>"
    else:
        alg = push_bytes
        achieved = push_gbs
        kname = push_kernel
    traffic = measured_traffic(args.config, kname, inner_per_step if dom == "solve" else t["n"])
    push_traffic = measured_traffic(args.config, push_kernel, t["n"])
    line = {
        "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world_size,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32 particles, f32 PCG under a double-float Newton residual",
        "data": "synthetic",
        "config": {"workload": args.config, "grid": list(cfg["n"]), "particles": int(t["n"]),
                   "initial_state": "GPU thermal loader" if big else "host synthetic",
                   "mpw0": cfg["mpw0"], "sort_every": cfg["sort_every"], "parallelism": "replicas",
                   "l2": "flushed between timed steps (256 MB write, outside the events)"},
        "poisson_ms_per_step": phases["solve"],
        "phase_ms_per_step": phases,
        "newton_per_step": t["newton"] / args.steps, "pcg_iterations_per_step": inner_per_step,
        "phi_rel_err_vs_fp64": err, "fp64_reference_converged": conv64,
        "errors_vs_fp64_oracle": errs,
        "reference_algorithm_iterations_per_step": ref_it,
        "fp64": fp64,
        "speedup_mixed_vs_fp64": (value / fp64["value"]) if fp64 else None,
        "e2e": {"value": e["n"] * world_size / (e["seconds"] / e2e_n), "unit": "particle-steps/s",
                "h2d_bytes_per_step": e["h2d"], "d2h_bytes_per_step": e["d2h"]},
        "gpu_launches": t["launches"],
        "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "peak_kind": peak_kind,
                     "algorithmic_bytes_per_launch": alg},
        "roofline_push": {"bound": "hbm", "kernel": push_kernel, "achieved": push_gbs, "peak": hbm,
                          "unit": "GB/s", "frac": push_gbs / hbm, "bytes_per_particle": 56,
                          "traffic": push_traffic},
        "clocks": ck,
    }
    # the step fuses the deposit into the push; alone, on the same ions: the
    # key and offsets read (16 B an ion), the accumulator cleared, read, and
    # turned into den with the node volumes (40 B a node)
    nn_all = int(np.prod(cfg["n"]))
    dep_bytes = 16.0 * t["n"] + 40.0 * nn_all
    dep_gbs = dep_bytes / (dep_ms * 1e-3) / 1e9
    line["roofline_deposit"] = {"bound": "hbm", "kernel": "k_deposit_tiles (espic_deposit: the clear, "
                                "k_deposit_tiles and k_deposit_tail, k_density)", "achieved": dep_gbs, "peak": hbm,
                                "unit": "GB/s",
                                "frac": dep_gbs / hbm, "ms": dep_ms, "bytes_per_particle": 16,
                                "bytes_per_node": 40}
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        if big:
            # a bounded sample: per-particle and per-iteration host costs,
            # measured, times this state's ion count and the reference
            # algorithm's iterations measured above
            c = cpu_sample_costs(cfg, 20_000_000, threads)
            step_s = t["n"] * c["pd_per_particle"] + ref_it["newton"] * c["newton_res_s"] + \
                ref_it["pcg"] * c["pcg_iter_s"]
            b = {"value": t["n"] / step_s,
                 "sample": "threaded push+removal+deposit of a 20M-ion sample (%d threads) scaled to %d ions; serial "
                           "Newton-PCG costs on the full grid (residual %.3f s, Jacobi-PCG iteration %.3f s) x the "
                           "reference algorithm's iterations for this state (%d Newton, %d Jacobi-PCG, measured on "
                           "the GPU above)" % (threads, int(t["n"]), c["newton_res_s"], c["pcg_iter_s"],
                                               ref_it["newton"], ref_it["pcg"])}
        else:
            r = cpu_sphere_steps(cfg, P0, threads, steps=2, warmup=1)
            b = {"value": r["n"] / r["seconds"],
                 "sample": "2 whole steps after 1 warm-up step on the host (%d threads for the particles, serial "
                           "Newton-PCG: %.2f Newton and %.1f Jacobi-PCG iterations per step, measured)"
                           % (threads, r["newton"], r["pcg"])}
        line["cpu_baseline"] = {"value": b["value"], "unit": "particle-steps/s", "cores": threads, "kind": "port",
                                "sample": b["sample"]}
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
