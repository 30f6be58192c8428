"""Generate the golden vectors in tests/golden/ by running the reference's own
CPU code (ch2, ch3/ver2, ch4, compiled from its sources by
oracle/build_ref.py) on seeded inputs.

Run here, where the reference checkout exists:
    python tests/golden/make_golden.py [base] [steady] [dsmc] [neutral] [ch4push] [ch4ion] [ionize]
The .npz files it writes are committed; the GPU host never needs the
reference.  Every fixture stores its inputs next to the reference outputs.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))
from oracle import build_ref, pyoracle as po  # noqa: E402
import steady_stats as ss  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
QE, AMU, ME, K = 1.602176565e-19, 1.660538921e-27, 9.10938215e-31, 1.380648e-23

BOX = dict(grid=[21, 21, 21], x0=[-0.1, -0.1, 0.0], xm=[0.1, 0.1, 0.2])
SPH = dict(grid=[21, 21, 41], x0=[-0.1, -0.1, 0.0], xm=[0.1, 0.1, 0.4])
SPHERE = [0.0, 0.0, 0.15, 0.05, -100.0]


def save(name, **arrays):
    path = os.path.join(OUT, name + ".npz")
    np.savez_compressed(path, **{k: np.asarray(v) for k, v in arrays.items()})
    print("wrote", path, os.path.getsize(path))


def rand_particles(rng, geo, n, vscale, wall_frac=0.1, w=1e4):
    x0, xm = np.array(geo["x0"]), np.array(geo["xm"])
    pos = x0 + rng.random((n, 3)) * (xm - x0)
    nw = int(n * wall_frac)
    # a share of the particles sits within a few steps of a wall
    axis = rng.integers(0, 3, nw)
    side = rng.integers(0, 2, nw)
    eps = rng.random(nw) * 3e-4
    for m in range(nw):
        a = axis[m]
        pos[m, a] = (x0[a] + eps[m]) if side[m] == 0 else (xm[a] - 1e-12 - eps[m])
    vel = (rng.random((n, 3)) * 2 - 1) * vscale
    P = np.zeros((7, n))
    P[0:3] = pos.T
    P[3:6] = vel.T
    P[6] = w * (0.5 + rng.random(n))
    return P


def base_inputs(geo, dt=0.0, **kw):
    d = dict(grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], dt=[dt])
    d.update(kw)
    return d


def smooth_phi(geo, rng, amp):
    ni, nj, nk = geo["grid"]
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    phi = amp * (np.sin(np.pi * i / (ni - 1)) * np.sin(np.pi * j / (nj - 1)) *
                 np.sin(2 * np.pi * k / (nk - 1) + 0.3))
    phi += amp * 0.01 * rng.standard_normal(phi.shape)
    return phi.ravel()


def box_cases(rng):
    g = po.grid(BOX["grid"], BOX["x0"], BOX["xm"])
    vol = po.run_reference("ref_ch2", "node_vol", base_inputs(BOX))["node_vol"]
    phi = smooth_phi(BOX, rng, 30.0)
    ef = po.efield(g, phi)
    dt = 2e-10
    Pi = rand_particles(rng, BOX, 1200, 2e4, w=1e4)
    Pe = rand_particles(rng, BOX, 800, 2e6, w=1e4)
    inp = base_inputs(BOX, dt, ns=[2], sp0_mq=[16 * AMU, QE], sp1_mq=[ME, -QE], sp0_P=Pi,
                      sp1_P=Pe, ef=ef.ravel())
    out = po.run_reference("ref_ch2", "push", inp)
    save("box_push", phi=phi, dt=dt, Pi=Pi, Pe=Pe,
         Pi_out=out["sp0_P"].reshape(7, -1), Pe_out=out["sp1_P"].reshape(7, -1), node_vol=vol)

    out = po.run_reference("ref_ch2", "deposit", inp)
    den_i, den_e = out["sp0_den"], out["sp1_den"]
    save("box_deposit", Pi=Pi, Pe=Pe, den_i=den_i, den_e=den_e, node_vol=vol)

    rinp = base_inputs(BOX, ns=[2], sp0_mq=[16 * AMU, QE], sp1_mq=[ME, -QE], sp0_den=den_i,
                       sp1_den=den_e)
    rho = po.run_reference("ref_ch2", "charge", rinp)["rho"]
    save("box_charge", den_i=den_i, den_e=den_e, rho=rho)

    phi0 = np.zeros(g.nn)
    sor = {}
    for tag, tol in (("c1", 1e-4), ("tight", 1e-9)):
        o = po.run_reference("ref_ch2", "sor", base_inputs(BOX, phi=phi0, rho=rho, max_it=[200000],
                                                           tol=[tol]))
        sor["phi_" + tag] = o["phi"]
        sor["conv_" + tag] = o["conv"]
    # a warm start: a perturbed phi, few iterations allowed
    warm = sor["phi_c1"] * 0.9
    o = po.run_reference("ref_ch2", "sor", base_inputs(BOX, phi=warm, rho=rho, max_it=[30],
                                                       tol=[1e-30]))
    save("box_sor", rho=rho, phi_warm=warm, phi_warm30=o["phi"], tol_c1=1e-4, tol_tight=1e-9,
         **sor)

    o = po.run_reference("ref_ch2", "efield", base_inputs(BOX, phi=phi))
    save("box_efield", phi=phi, ef=o["ef"].reshape(-1, 3))

    o = po.run_reference("ref_ch2", "diag", inp)
    save("box_diag", Pi=Pi, Pe=Pe, phi=phi, mi=16 * AMU, me=ME, diag_i=o["sp0_diag"],
         diag_e=o["sp1_diag"], pe=o["pe"])

    # random and quiet-start loaders (uniforms of the reference's mt19937 recorded)
    linp = base_inputs(BOX, dt, ns=[1], sp0_mq=[16 * AMU, QE], ef=ef.ravel(), seed=[1234],
                       x1=BOX["x0"], x2=BOX["xm"], num_den=[1e11], num_mp=[3000])
    o = po.run_reference("ref_ch2", "load_box", linp)
    qinp = base_inputs(BOX, dt, ns=[1], sp0_mq=[ME, -QE], ef=ef.ravel(), x1=BOX["x0"],
                       x2=[0.0, 0.0, 0.1], num_den=[1e11], num_mp=[11, 9, 13])
    q = po.run_reference("ref_ch2", "load_qs", qinp)
    save("box_load", phi=phi, dt=dt, u=o["u"], P_box=o["sp0_P"].reshape(7, -1),
         P_qs=q["sp0_P"].reshape(7, -1), num_mp_box=3000, num_mp_qs=[11, 9, 13],
         qs_x2=[0.0, 0.0, 0.1])

    # a short run of the ch2 main loop: 80,000/10,000 scaled down to 3,000/600
    sinp = base_inputs(BOX, dt, ns=[1], sp0_mq=[16 * AMU, QE], seed=[77], x1=BOX["x0"],
                       x2=BOX["xm"], num_den=[1e11], num_mp=[3000], ef=np.zeros(3 * g.nn))
    li = po.run_reference("ref_ch2", "load_box", sinp)
    sinp2 = base_inputs(BOX, dt, ns=[1], sp0_mq=[ME, -QE], seed=[78], x1=BOX["x0"],
                        x2=[0.0, 0.0, 0.1], num_den=[1e11], num_mp=[600], ef=np.zeros(3 * g.nn))
    le = po.run_reference("ref_ch2", "load_box", sinp2)
    Pi0 = li["sp0_P"].reshape(7, -1)
    Pe0 = le["sp0_P"].reshape(7, -1)
    st = base_inputs(BOX, dt, steps=[40], ns=[2], sp0_mq=[16 * AMU, QE], sp1_mq=[ME, -QE],
                     sp0_P=Pi0, sp1_P=Pe0, max_it=[10000], tol=[1e-4], initial_solve=[1])
    o = po.run_reference("ref_ch2", "steps", st)
    save("box_steps", Pi0=Pi0, Pe0=Pe0, ui=li["u"], ue=le["u"], dt=dt, steps=40,
         hist=o["hist"].reshape(41, -1), phi=o["phi"], Pi=o["sp0_P"].reshape(7, -1),
         Pe=o["sp1_P"].reshape(7, -1))


def sphere_cases(rng):
    g = po.grid(SPH["grid"], SPH["x0"], SPH["xm"])
    o = po.run_reference("ref_ch3", "objects", base_inputs(SPH, sphere=SPHERE, inlet=[1]))
    obj, phi_obj = o["object_id"], o["phi"]
    save("sphere_objects", object_id=obj, phi=phi_obj, sphere=SPHERE)

    dt = 1e-7
    mi = 16 * AMU
    phi = smooth_phi(SPH, rng, 20.0)
    phi[obj > 0] = phi_obj[obj > 0]
    ef = po.efield(g, phi)
    # ions: bulk, near walls, near the sphere surface
    P = rand_particles(rng, SPH, 1500, 4e4, wall_frac=0.15, w=50.0)
    ns_ = 300
    d = rng.standard_normal((ns_, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    r = 0.05 + rng.random(ns_) * 4e-3
    P[0:3, :ns_] = (np.array(SPHERE[:3]) + d * r[:, None]).T
    P[3:6, :ns_] = (-d * 4e4).T
    inp = base_inputs(SPH, dt, ns=[1], sp0_mq=[mi, QE, 50.0], sp0_P=P, ef=ef.ravel(),
                      sphere=SPHERE, inlet=[1])
    o = po.run_reference("ref_ch3", "push_sphere", inp)
    save("sphere_push", phi=phi, dt=dt, P=P, P_out=o["sp0_P"].reshape(7, -1))

    o = po.run_reference("ref_ch3", "deposit", inp)
    vol = po.node_volumes(g)
    save("sphere_deposit", P=P, den=o["sp0_den"], node_vol=vol)
    rho = o["sp0_den"] * QE

    ref = [0.0, 3.0, 1e10]
    gs = {}
    for tag, tol, mx in (("c2", 1e-4, 20000), ("tight", 1e-9, 400000)):
        o = po.run_reference("ref_ch3", "gs", base_inputs(SPH, sphere=SPHERE, inlet=[1], rho=rho,
                                                          ref=ref, max_it=[mx], tol=[tol]))
        gs["phi_" + tag] = o["phi"]
        gs["conv_" + tag] = o["conv"]
    o = po.run_reference("ref_ch3", "qn", base_inputs(SPH, sphere=SPHERE, inlet=[1], rho=rho,
                                                      ref=ref, max_it=[1], tol=[1.0]))
    save("sphere_solve", rho=rho, object_id=obj, phi_init=phi_obj, ref=ref, phi_qn=o["phi"], **gs)

    o = po.run_reference("ref_ch3", "efield", base_inputs(SPH, phi=phi))
    save("sphere_efield", phi=phi, ef=o["ef"].reshape(-1, 3))

    # cold beam injection (ColdBeamSource), uniforms recorded
    o = po.run_reference("ref_ch3", "inject_cold",
                         base_inputs(SPH, dt, ns=[1], sp0_mq=[mi, QE, 200.0], ef=ef.ravel(),
                                     seed=[4321], source=[7000.0, 1e10]))
    save("inject_cold", phi=phi, dt=dt, mpw0=200.0, v_drift=7000.0, den=1e10, u=o["u"],
         P=o["sp0_P"].reshape(7, -1))
    # warm beam injection (ch4 WarmBeamSource), T_i = 0.1 eV
    T = 0.1 * QE / K
    o = po.run_reference("ref_ch4", "inject_warm",
                         base_inputs(SPH, dt, sp0_mq=[mi, QE, 200.0], ef=ef.ravel(), seed=[999],
                                     source=[7000.0, 1e10, T]))
    save("inject_warm", phi=phi, dt=dt, mpw0=200.0, v_drift=7000.0, den=1e10, temp=T, u=o["u"],
         P=o["sp0_P"].reshape(7, -1))

    dens = rng.random((3, g.nn)) * 1e10
    o = po.run_reference("ref_ch3", "update_average",
                         base_inputs(SPH, ns=[1], sp0_mq=[mi, QE, 5.0], dens=dens.ravel()))
    save("update_average", dens=dens, den_ave=o["den_ave"])

    # a short run of the ch3/ver2 main loop (ColdBeamSource, solveGS)
    st = base_inputs(SPH, dt, steps=[30], ns=[1], sp0_mq=[mi, QE, 5e2], seed=[2024],
                     sphere=SPHERE, inlet=[1], source=[7000.0, 1e10], ref=[0.0, 1.5, 1e10],
                     max_it=[20000], tol=[1e-4], initial_solve=[1])
    o = po.run_reference("ref_ch3", "steps", st)
    save("sphere_steps", hist=o["hist"].reshape(31, -1), u=o["u"], u_count=o["u_count"],
         phi=o["phi"], P=o["sp0_P"].reshape(7, -1), den=o["sp0_den"], steps=30, dt=dt,
         mpw0=5e2)


def dsmc_cases():
    """Three DSMC_MEX::apply calls (ch4/Collisions.cpp:108-183) on 3000 oxygen
    atoms in 125 cells: a 7 km/s beam with anisotropic thermal spread, specific
    weight 1e14, the reference's starting sigma_cr_max (1e-14)."""
    geo = dict(grid=[6, 6, 6], x0=[0.0, 0.0, 0.0], xm=[0.05, 0.05, 0.05])
    rng = np.random.default_rng(20261204)
    n, mass, mpw0, dt = 3000, 16 * AMU, 1e14, 1e-7
    P = np.zeros((7, n))
    P[0:3] = rng.random((3, n)) * 0.05 * 0.999999
    P[3] = 7000 + 300 * rng.standard_normal(n)
    P[4] = 300 * rng.standard_normal(n)
    P[5] = 150 * rng.standard_normal(n)
    P[6] = mpw0
    o = po.run_reference("ref_ch4", "dsmc", base_inputs(geo, dt, seed=[77], sp0_mq=[mass, 0.0, mpw0],
                                                        sp0_P=P.ravel(), steps=[3]))
    save("dsmc_steps", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], mass=mass, mpw0=mpw0, dt=dt, P0=P,
         P=o["sp0_P"].reshape(7, -1), u=o["u"], sigma_cr_max=o["sigma_cr_max"], c=o["c"])


def neutral_cases():
    """ch4 species moments (Species::sampleMoments twice, computeGasProperties,
    computeMPC, ch4/Species.cpp:191-235) of 2000 weighted atoms, and two
    MCC_CEX::apply calls (ch4/Collisions.cpp:43-80) of 2000 ions in a given
    neutral gas (density 0.5-3e19 m^-3, stream velocity about 7 km/s)."""
    geo = dict(grid=[6, 6, 6], x0=[0.0, 0.0, 0.0], xm=[0.05, 0.05, 0.05])
    rng = np.random.default_rng(20261205)
    n, mass = 2000, 16 * AMU
    P = np.zeros((7, n))
    P[0:3] = rng.random((3, n)) * 0.05 * 0.999999
    P[3] = 7000 + 500 * rng.standard_normal(n)
    P[4] = 200 * rng.standard_normal(n)
    P[5] = -300 + 400 * rng.standard_normal(n)
    P[6] = 1e12 * (0.5 + rng.random(n))
    o = po.run_reference("ref_ch4", "moments", base_inputs(geo, 1e-7, seed=[5], sp0_mq=[mass, 0.0, 1e12],
                                                           sp0_P=P.ravel(), calls=[2]))
    save("neutral_moments", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], mass=mass, calls=2, P=P,
         mom=o["mom"], vel=o["vel"], T=o["T"], mpc=o["mpc"])
    nn = int(np.prod(geo["grid"]))
    X = np.stack(np.meshgrid(*[np.linspace(geo["x0"][d], geo["xm"][d], geo["grid"][d]) for d in range(3)],
                             indexing="ij"), axis=-1).transpose(2, 1, 0, 3).reshape(nn, 3)
    den = 1e19 * (1.75 + 1.25 * np.sin(X[:, 0] * 90) * np.cos(X[:, 2] * 60))
    vel = np.zeros((nn, 3))
    vel[:, 2] = 7000 + 300 * np.sin(X[:, 1] * 70)
    vel[:, 0] = 100 * rng.standard_normal(nn)
    T = 1000 + 50 * rng.random(nn)
    Pi = np.zeros((7, n))
    Pi[0:3] = rng.random((3, n)) * 0.05 * 0.999999
    Pi[3:6] = 2000 * rng.standard_normal((3, n))
    Pi[6] = 5e2
    dt = 1e-8
    o = po.run_reference("ref_ch4", "mcc", base_inputs(geo, dt, seed=[41], sp0_mq=[mass, QE, 5e2], sp0_P=Pi.ravel(),
                                                       sp1_mq=[mass, 0.0, 1e12], sp1_den=den, sp1_vel=vel.ravel(),
                                                       sp1_T=T, steps=[2]))
    save("neutral_mcc", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], dt=dt, P0=Pi, den=den, vel=vel.ravel(),
         T=T, u=o["u"], P=o["sp0_P"].reshape(7, -1), steps=2)


def ch4_push_cases():
    """Five Species::advance(neutrals, neutrals) steps (ch4/Species.cpp:8-91)
    of 3000 oxygen atoms flowing at 7 km/s past the sphere: diffuse
    reflection off its surface at the 1000 K wall speed, removal at the
    domain faces; half of the atoms start with a full step of time left (as
    a source leaves them), half with none."""
    geo = SPH
    rng = np.random.default_rng(20261206)
    n, mass, dt = 3000, 16 * AMU, 2e-6
    x0, xm = np.array(geo["x0"]), np.array(geo["xm"])
    P = np.zeros((7, n))
    c = np.array(SPHERE[:3])
    pos = x0 + rng.random((3 * n, 3)) * (xm - x0)
    pos = pos[np.sum((pos - c) ** 2, axis=1) > (SPHERE[3] + 1e-3) ** 2][:n]
    P[0:3] = pos.T
    P[3:6] = 300 * rng.standard_normal((3, n))
    P[5] += 7000
    P[6] = 1e12
    pdt = np.where(rng.random(n) < 0.5, dt, 0.0)
    o = po.run_reference("ref_ch4", "advance", base_inputs(geo, dt, seed=[13], sp0_mq=[mass, 0.0, 1e12],
                                                           sp0_P=P.ravel(), sp0_dt=pdt, sphere=SPHERE, steps=[5]))
    save("ch4_push", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], mass=mass, dt=dt, sphere=SPHERE, P0=P,
         dt0=pdt, steps=5, u=o["u"], P=o["sp0_P"].reshape(7, -1), pdt=o["sp0_dt"])


def ch4_ion_push_cases():
    """Three Species::advance(neutrals, neutrals) steps of 1500 O+ ions
    (ch4/Species.cpp:8-91) in a given E field: ions striking the sphere are
    removed and leave two neutrals each (mpw0 ratio 2) and, above 5000 m/s,
    a sputtered atom with probability 0.2."""
    geo = SPH
    rng = np.random.default_rng(20261207)
    n, mass, dt = 1500, 16 * AMU, 2e-6
    x0, xm = np.array(geo["x0"]), np.array(geo["xm"])
    c = np.array(SPHERE[:3])
    pos = x0 + rng.random((3 * n, 3)) * (xm - x0)
    pos = pos[np.sum((pos - c) ** 2, axis=1) > (SPHERE[3] + 1e-3) ** 2][:n]
    P = np.zeros((7, n))
    P[0:3] = pos.T
    P[3:6] = 600 * rng.standard_normal((3, n))
    P[5] += 6000
    P[6] = 2e11
    nn = int(np.prod(geo["grid"]))
    ef = 200 * rng.standard_normal((nn, 3))
    pdt = np.where(rng.random(n) < 0.5, dt, 0.0)
    o = po.run_reference("ref_ch4", "advance_ion", base_inputs(geo, dt, seed=[17], sp0_mq=[mass, QE, 2e11],
                                                               sp0_P=P.ravel(), sp0_dt=pdt, sp1_mq=[mass, 0.0, 1e11],
                                                               sphere=SPHERE, ef=ef.ravel(), steps=[3]))
    save("ch4_ion_push", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], mass=mass, charge=QE, mpw0=2e11, dt=dt,
         sphere=SPHERE, ef=ef.ravel(), P0=P, dt0=pdt, steps=3, neutral=[1e11, 0.0, mass], u=o["u"],
         P=o["sp0_P"].reshape(7, -1), pdt=o["sp0_dt"], N=o["sp1_P"].reshape(7, -1), ndt=o["sp1_dt"])


def ionize_cases():
    """ChemistryIonize::apply (ch4/Collisions.cpp:10-31) on a 11x11x21 grid:
    neutral density 1e16-1e17 m^-3, rho of a 1e13-1e14 m^-3 plasma, rate
    5e-11 m^3/s (about one ion per cell), ion weight 1e8, an E field for the
    velocity rewind."""
    geo = dict(grid=[11, 11, 21], x0=[-0.1, -0.1, 0.0], xm=[0.1, 0.1, 0.4])
    rng = np.random.default_rng(20261208)
    nn = int(np.prod(geo["grid"]))
    den = 1e16 * (1 + 9 * rng.random(nn))
    rho = QE * 1e13 * (1 + 9 * rng.random(nn))
    ef = 100 * rng.standard_normal((nn, 3))
    mass, mpw0, rate, dt = 16 * AMU, 1e8, 5e-11, 1e-7
    o = po.run_reference("ref_ch4", "ionize", base_inputs(geo, dt, seed=[19], sp0_mq=[mass, QE, mpw0],
                                                          sp1_mq=[mass, 0.0, 1e12], sp1_den=den, rho=rho,
                                                          ef=ef.ravel(), rate=[rate]))
    save("ch4_ionize", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], mass=mass, charge=QE, mpw0=mpw0, rate=rate,
         dt=dt, den=den, rho=rho, ef=ef.ravel(), u=o["u"], P=o["sp0_P"].reshape(7, -1), pdt=o["sp0_dt"])


def dsmc_sparse_cases():
    """DSMC_MEX::apply on 300 atoms in 125 cells (0 to ~6 per cell): cells
    too small to pair, and two-atom cells where the second pick is redrawn
    until it differs from the first (ch4/Collisions.cpp:148-152), five calls
    from the reference's starting sigma_cr_max."""
    geo = dict(grid=[6, 6, 6], x0=[0.0, 0.0, 0.0], xm=[0.05, 0.05, 0.05])
    rng = np.random.default_rng(20261209)
    n, mass, mpw0, dt = 300, 16 * AMU, 1e15, 1e-6
    P = np.zeros((7, n))
    P[0:3] = rng.random((3, n)) * 0.05 * 0.999999
    P[3:6] = 500 * rng.standard_normal((3, n))
    P[6] = mpw0
    o = po.run_reference("ref_ch4", "dsmc", base_inputs(geo, dt, seed=[78], sp0_mq=[mass, 0.0, mpw0],
                                                        sp0_P=P.ravel(), steps=[5]))
    save("dsmc_sparse", grid=geo["grid"], x0=geo["x0"], xm=geo["xm"], mass=mass, mpw0=mpw0, dt=dt, P0=P,
         P=o["sp0_P"].reshape(7, -1), u=o["u"], sigma_cr_max=o["sigma_cr_max"], c=o["c"], steps=5)


def steady_run(seed):
    """One 600-step run of the ch3/ver2 main loop at the reference's own
    macroparticle weight (ch3/ver2/Main.cpp:33), with batch means of den and
    phi over time steps 200-599 and the reference's den_ave."""
    st = base_inputs(SPH, ss.DT, steps=[ss.STEPS], ns=[1], sp0_mq=[16 * AMU, QE, ss.MPW0], seed=[seed],
                     sphere=SPHERE, inlet=[1], source=[7000.0, 1e10], ref=[0.0, 1.5, 1e10],
                     max_it=[20000], tol=[1e-4], initial_solve=[1], avg=list(ss.AVG))
    o = po.run_reference("ref_ch3", "steps", st)
    hist = o["hist"].reshape(-1, 9)     # ts, np, real count, momentum (3), KE, PE, steady
    nb = ss.AVG[2]
    out = ss.batch_profiles(o["sp0_den_batches"].reshape(nb, -1), o["phi_batches"].reshape(nb, -1))
    tot = np.zeros((nb, 3))
    for row in hist:
        b = ss.batch_index(int(row[0]))
        if b >= 0:
            tot[b] += row[[1, 6, 7]] / ss.AVG[1]
    out["totals"] = tot
    ave = ss.profiles(o["sp0_den_ave"], o["phi"])
    out.update({"ave_" + k: ave[k] for k in ("axial", "wake", "radial")})
    out["steady_ts"] = hist[np.nonzero(hist[:, 8])[0][0], 0]
    return out


def steady_cases():
    """Steady-state statistics of the sphere run, two seeds (run concurrently)."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(2) as ex:
        runs = list(ex.map(steady_run, (1, 2)))
    arrays = {}
    for seed, r in zip((1, 2), runs):
        arrays.update({"%s_s%d" % (k, seed): v for k, v in r.items()})
    save("sphere_steady", steps=ss.STEPS, dt=ss.DT, mpw0=ss.MPW0, avg=np.array(ss.AVG), **arrays)


def ch9mpi_source_cases(rng):
    """Five calls of the particle source of the ch9/MPI variant
    (ch9/MPI/src/Source.cpp:5-72, compiled with a stand-in mpi.h): fixed-
    speed isotropic velocities, v_z < 0 reflected, the macroparticle count's
    fraction carried between calls, velocities rewound in a smooth E."""
    g = po.grid(SPH["grid"], SPH["x0"], SPH["xm"])
    phi = smooth_phi(SPH, rng, 40.0)
    ef = po.efield(g, phi)
    dt, spwt, den0, v_drift, T = 1e-7, 3.1e3, 1e10, 7000.0, 0.1 * QE / K
    inp = dict(grid=SPH["grid"], x0=SPH["x0"], dh=list(g.dh), dt=[dt], ef=ef.ravel(), seed=[4242],
               species=[16 * AMU, QE, spwt, 5000], source=[den0, v_drift, T], calls=[5])
    o = po.run_reference("ref_ch9mpi", "sample", inp)
    n = int(o["counts"].sum())
    save("inject_ch9mpi", phi=phi, dt=dt, spwt=spwt, den0=den0, v_drift=v_drift, T=T, P=o["P"].reshape(7, n),
         counts=o["counts"], rem=o["rem"], used=o["used"], u=o["u"], v_th=o["v_th"])


LONG_STEPS, LONG_BATCH, LONG_SEEDS = 10000, 500, (1, 2, 3, 4, 5, 6)


def box_longrun(seed):
    """One 10,000-step run of the ch2 main loop at the reference's
    configuration 1 (80,000 O+ over the box and 10,000 electrons in the
    octant [-0.1,0]^2 x [0,0.1] at n = 1e11, ch2/snippets/step4/Main.cpp:31-34;
    dt 2e-10; SOR to 1e-4, ch2/Main.cpp:38): the energy history
    (ch2/Output.cpp:82-118 columns) reduced to batch means."""
    g = po.grid(BOX["grid"], BOX["x0"], BOX["xm"])
    dt = 2e-10
    li = po.run_reference("ref_ch2", "load_box", base_inputs(
        BOX, dt, ns=[1], sp0_mq=[16 * AMU, QE], seed=[1000 + seed], x1=BOX["x0"], x2=BOX["xm"],
        num_den=[1e11], num_mp=[80000], ef=np.zeros(3 * g.nn)))
    le = po.run_reference("ref_ch2", "load_box", base_inputs(
        BOX, dt, ns=[1], sp0_mq=[ME, -QE], seed=[2000 + seed], x1=BOX["x0"], x2=[0.0, 0.0, 0.1],
        num_den=[1e11], num_mp=[10000], ef=np.zeros(3 * g.nn)))
    st = base_inputs(BOX, dt, steps=[LONG_STEPS], ns=[2], sp0_mq=[16 * AMU, QE], sp1_mq=[ME, -QE],
                     sp0_P=li["sp0_P"], sp1_P=le["sp0_P"], max_it=[10000], tol=[1e-4], initial_solve=[1])
    # one row per time step (the loop runs while ts <= num_ts: steps + 1 rows);
    # columns: ts, then per species np, real count, px, py, pz, KE; then PE
    h = po.run_reference("ref_ch2", "steps", st)["hist"].reshape(-1, 14)[:LONG_STEPS]
    return np.stack([h[:, 6], h[:, 12], h[:, 13], h[:, 6] + h[:, 12] + h[:, 13]], axis=1)


def box_longrun_cases():
    """Energy history of configuration 1 from several seeds of the
    reference's own loop (run concurrently): batch means of KE (ions,
    electrons), PE and their sum over 500-step batches, and the full
    history of the first 200 steps."""
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(len(LONG_SEEDS)) as ex:
        runs = list(ex.map(box_longrun, LONG_SEEDS))
    E = np.stack(runs)  # [seed][step][KE_i, KE_e, PE, total]
    nb = LONG_STEPS // LONG_BATCH
    batches = E.reshape(len(LONG_SEEDS), nb, LONG_BATCH, 4).mean(axis=2)
    save("box_longrun", steps=LONG_STEPS, batch=LONG_BATCH, seeds=np.array(LONG_SEEDS), batches=batches,
         early=E[:, :200, :])


if __name__ == "__main__":
    # optional arguments select cases: "base" (box and sphere, one random
    # stream), "steady", "dsmc", "neutral", "ch4push", "ch4ion", "ionize" (default: all)
    cases = sys.argv[1:] or ["base", "steady", "dsmc", "neutral", "ch4push", "ch4ion", "ionize"]
    build_ref.build_reference()
    if "base" in cases:
        rng = np.random.default_rng(20261203)
        box_cases(rng)
        sphere_cases(rng)
    if "steady" in cases:
        steady_cases()
    if "dsmc" in cases:
        dsmc_cases()
        dsmc_sparse_cases()
    if "neutral" in cases:
        neutral_cases()
    if "ch4push" in cases:
        ch4_push_cases()
    if "ch4ion" in cases:
        ch4_ion_push_cases()
    if "ionize" in cases:
        ionize_cases()
    if "longrun" in cases:
        box_longrun_cases()
    if "ch9mpi" in cases:
        ch9mpi_source_cases(np.random.default_rng(909))
