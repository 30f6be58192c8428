"""Pins the CPU oracle to the reference: every restated function against the
golden vectors produced by the reference's own code (tests/golden/)."""
import numpy as np
import pytest

from conftest import golden

QE, AMU, ME, K = 1.602176565e-19, 1.660538921e-27, 9.10938215e-31, 1.380648e-23
BOX = ([21, 21, 21], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.2])
SPH = ([21, 21, 41], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.4])
SPHERE4 = [0.0, 0.0, 0.15, 0.05 * 0.05]


def test_node_volumes(po):
    g = po.grid(*BOX)
    assert np.array_equal(po.node_volumes(g), golden("box_push")["node_vol"])


def test_box_push_bitexact(po):
    f = golden("box_push")
    g = po.grid(*BOX)
    ef = po.efield(g, f["phi"])
    Pi = po.push_box(g, ef, QE, 16 * AMU, float(f["dt"]), f["Pi"])
    Pe = po.push_box(g, ef, -QE, ME, float(f["dt"]), f["Pe"])
    assert np.array_equal(Pi, f["Pi_out"])
    assert np.array_equal(Pe, f["Pe_out"])
    # the fixture exercises the wall reflections
    assert np.any(np.sign(f["Pe"][3:6]) != np.sign(f["Pe_out"][3:6]))


def test_box_deposit(po):
    f = golden("box_deposit")
    g = po.grid(*BOX)
    vol = f["node_vol"]
    for P, den in ((f["Pi"], f["den_i"]), (f["Pe"], f["den_e"])):
        # the reference's own FP64 sum, restated: bit-exact
        assert np.array_equal(po.divide_volume(po.deposit_fp64(g, P), vol), den)
        # the fixed-point deposit: one rounding per corner weight, so a node
        # holding c contributions is off by at most c/2 quanta (2^-S each),
        # plus the reference's own FP64 summation error
        S = po.fixed_scale_exponent(float(P[6].max()), 10**6)
        fx = 2.0**S
        acc = po.deposit_fixed(g, P, fx)
        d2 = po.density_from_fixed(acc, fx, vol)
        contrib = po.deposit_fixed(g, np.vstack([P[:6], np.ones((1, P.shape[1]))]), 1.0)
        bound = (0.5 * (contrib + 8) / fx + 1e-15 * np.abs(den) * vol * 64) / vol
        assert np.all(np.abs(d2 - den) <= bound)
        assert np.max(np.abs(d2 - den)) <= 1e-12 * np.max(np.abs(den))


def test_fixed_scale_exponent(po):
    S = po.fixed_scale_exponent(1e4, 10**6)
    assert 1e6 * 1e4 * 2.0**S <= 2.0**62 < 1e6 * 1e4 * 2.0**(S + 1)
    assert po.fixed_scale_exponent(1e-30, 1) == 52


def test_charge_density(po):
    f = golden("box_charge")
    rho = po.charge_density([QE, -QE], np.stack([f["den_i"], f["den_e"]]))
    assert np.array_equal(rho, f["rho"])
    # neutrals are skipped
    rho0 = po.charge_density([QE, 0.0], np.stack([f["den_i"], f["den_e"]]))
    assert np.array_equal(rho0, po.charge_density([QE], f["den_i"][None]))


def test_box_sor_lex_bitexact(po):
    f = golden("box_sor")
    g = po.grid(*BOX)
    for tag, tol in (("c1", 1e-4), ("tight", 1e-9)):
        phi, conv, l2, it = po.sor_box(g, np.zeros(g.nn), f["rho"], 200000, tol, order="lex")
        assert conv and bool(f["conv_" + tag][0])
        assert np.array_equal(phi, f["phi_" + tag])
    phi, conv, _, it = po.sor_box(g, f["phi_warm"], f["rho"], 30, 1e-30, order="lex")
    assert not conv and it == 30
    assert np.array_equal(phi, f["phi_warm30"])


def test_box_sor_redblack_converges_to_reference(po):
    f = golden("box_sor")
    g = po.grid(*BOX)
    phi, conv, l2, it = po.sor_box(g, np.zeros(g.nn), f["rho"], 200000, 1e-9, order="rb")
    assert conv and l2 < 1e-9
    ref = f["phi_tight"]
    assert np.max(np.abs(phi - ref)) <= 1e-9 * np.max(np.abs(ref))


def test_efield_bitexact(po):
    for geo, name in ((BOX, "box_efield"), (SPH, "sphere_efield")):
        f = golden(name)
        g = po.grid(*geo)
        assert np.array_equal(po.efield(g, f["phi"]), f["ef"])


def test_diagnostics_bitexact(po):
    f = golden("box_diag")
    g = po.grid(*BOX)
    assert np.array_equal(po.species_diag(f["Pi"], float(f["mi"])), f["diag_i"])
    assert np.array_equal(po.species_diag(f["Pe"], float(f["me"])), f["diag_e"])
    ef = po.efield(g, f["phi"])
    assert po.potential_energy(g, ef, po.node_volumes(g)) == f["pe"][0]


def test_loaders_bitexact(po):
    f = golden("box_load")
    g = po.grid(*BOX)
    ef = po.efield(g, f["phi"])
    dt = float(f["dt"])
    P = po.load_box(g, ef, QE, 16 * AMU, dt, BOX[1], BOX[2], 1e11, 3000, f["u"])
    assert len(f["u"]) == 3 * 3000
    assert np.array_equal(P, f["P_box"])
    Q = po.load_box_qs(g, ef, -QE, ME, dt, BOX[1], f["qs_x2"], 1e11, f["num_mp_qs"])
    assert np.array_equal(Q, f["P_qs"])


def _box_step_oracle(po, g, vol, species, dt, phi, ef):
    for s in species:
        s["P"] = po.push_box(g, ef, s["q"], s["m"], dt, s["P"])
        s["den"] = po.divide_volume(po.deposit_fp64(g, s["P"]), vol)
    rho = po.charge_density([s["q"] for s in species], np.stack([s["den"] for s in species]))
    phi, _, _, _ = po.sor_box(g, phi, rho, 10000, 1e-4, order="lex")
    return phi, po.efield(g, phi)


def test_box_main_loop_bitexact(po):
    """41 iterations of the ch2 main loop restated from oracle pieces."""
    f = golden("box_steps")
    g = po.grid(*BOX)
    vol = po.node_volumes(g)
    dt = float(f["dt"])
    zero = np.zeros((g.nn, 3))
    sp = [dict(q=QE, m=16 * AMU, P=po.load_box(g, zero, QE, 16 * AMU, dt, BOX[1], BOX[2], 1e11,
                                                3000, f["ui"])),
          dict(q=-QE, m=ME, P=po.load_box(g, zero, -QE, ME, dt, BOX[1], [0.0, 0.0, 0.1], 1e11,
                                          600, f["ue"]))]
    assert np.array_equal(sp[0]["P"], f["Pi0"]) and np.array_equal(sp[1]["P"], f["Pe0"])
    phi, _, _, _ = po.sor_box(g, np.zeros(g.nn), np.zeros(g.nn), 10000, 1e-4, order="lex")
    ef = po.efield(g, phi)
    hist = f["hist"]
    for st in range(hist.shape[0]):
        phi, ef = _box_step_oracle(po, g, vol, sp, dt, phi, ef)
        row = [st]
        for s in sp:
            d = po.species_diag(s["P"], s["m"])
            row += [s["P"].shape[1], d[0], d[1], d[2], d[3], d[4]]
        row.append(po.potential_energy(g, ef, vol))
        assert np.array_equal(np.array(row), hist[st]), st
    assert np.array_equal(phi, f["phi"])
    assert np.array_equal(sp[0]["P"], f["Pi"]) and np.array_equal(sp[1]["P"], f["Pe"])


def test_sphere_objects_bitexact(po):
    f = golden("sphere_objects")
    g = po.grid(*SPH)
    obj, phi = po.objects(g, f["sphere"][:3], f["sphere"][3], f["sphere"][4])
    assert np.array_equal(obj, f["object_id"].astype(np.int32))
    assert np.array_equal(phi, f["phi"])


def test_sphere_push_bitexact(po):
    f = golden("sphere_push")
    g = po.grid(*SPH)
    ef = po.efield(g, f["phi"])
    P = po.push_sphere(g, ef, SPHERE4, QE, 16 * AMU, float(f["dt"]), f["P"])
    assert P.shape[1] < f["P"].shape[1]  # absorption happened
    assert np.array_equal(P, f["P_out"])
    # the CUDA path's compaction order keeps the same survivors
    H = po.push_sphere(g, ef, SPHERE4, QE, 16 * AMU, float(f["dt"]), f["P"], compact="holes")
    a = H[:, np.lexsort(H[:3])]
    b = P[:, np.lexsort(P[:3])]
    assert np.array_equal(a, b)


def test_sphere_deposit_bitexact(po):
    f = golden("sphere_deposit")
    g = po.grid(*SPH)
    assert np.array_equal(po.divide_volume(po.deposit_fp64(g, f["P"]), f["node_vol"]), f["den"])


def test_sphere_solvers(po):
    f = golden("sphere_solve")
    g = po.grid(*SPH)
    obj = f["object_id"].astype(np.int32)
    phi0, te0, n0 = f["ref"]
    phi, conv, l2, it = po.gs_sphere(g, f["phi_init"], f["rho"], obj, phi0, te0, n0, 20000, 1e-4,
                                     order="lex")
    assert conv and np.array_equal(phi, f["phi_c2"])
    assert np.array_equal(po.qn(g, f["phi_init"], f["rho"], obj, phi0, te0, n0), f["phi_qn"])
    ref = f["phi_tight"]
    scale = np.max(np.abs(ref))
    # the red-black form of solveGS reaches the same solution
    phi, conv, l2, it = po.gs_sphere(g, f["phi_init"], f["rho"], obj, phi0, te0, n0, 400000, 1e-9,
                                     order="rb")
    assert conv and np.max(np.abs(phi - ref)) <= 1e-8 * scale
    # and so does the symmetric Newton-PCG form
    phi, conv, nr, pcg = po.newton_pcg(g, f["phi_init"], f["rho"], obj, phi0, te0, n0, 30, 1e-12,
                                       20000, 1e-12)
    assert conv and np.max(np.abs(phi - ref)) <= 1e-8 * scale


def test_injection_bitexact(po):
    g = po.grid(*SPH)
    for name, temp in (("inject_cold", None), ("inject_warm", None)):
        f = golden(name)
        ef = po.efield(g, f["phi"])
        t = float(f["temp"]) if "temp" in f else None
        P, used = po.inject(g, ef, QE, 16 * AMU, float(f["dt"]), float(f["mpw0"]),
                            float(f["v_drift"]), float(f["den"]), f["u"], temp=t)
        assert used == len(f["u"])
        assert P.shape == f["P"].shape and P.shape[1] > 100
        assert np.array_equal(P, f["P"]), name


def test_update_average_bitexact(po):
    f = golden("update_average")
    ave = np.zeros(f["dens"].shape[1])
    for s, d in enumerate(f["dens"]):
        ave = po.update_average(ave, d, s)
    assert np.array_equal(ave, f["den_ave"])


def test_sphere_main_loop_bitexact(po):
    """31 iterations of the ch3/ver2 main loop (cold beam, solveGS)."""
    f = golden("sphere_steps")
    g = po.grid(*SPH)
    vol = po.node_volumes(g)
    obj, phi = po.objects(g, [0.0, 0.0, 0.15], 0.05, -100.0)
    dt, mpw0 = float(f["dt"]), float(f["mpw0"])
    m = 16 * AMU
    phi, _, _, _ = po.gs_sphere(g, phi, np.zeros(g.nn), obj, 0.0, 1.5, 1e10, 20000, 1e-4, "lex")
    ef = po.efield(g, phi)
    P = np.zeros((7, 0))
    u_all, counts = f["u"], f["u_count"].astype(int)
    off = 0
    steady = False
    last = np.zeros(3)
    for st in range(f["hist"].shape[0]):
        u = u_all[off:off + counts[st]]
        off += counts[st]
        P, used = po.inject(g, ef, QE, m, dt, mpw0, 7000.0, 1e10, u, P=P)
        assert used == counts[st]
        P = po.push_sphere(g, ef, SPHERE4, QE, m, dt, P)
        den = po.divide_volume(po.deposit_fp64(g, P), vol)
        rho = po.charge_density([QE], den[None])
        phi, _, _, _ = po.gs_sphere(g, phi, rho, obj, 0.0, 1.5, 1e10, 20000, 1e-4, "lex")
        ef = po.efield(g, phi)
        d = po.species_diag(P, m)
        pe = po.potential_energy(g, ef, vol)
        if not steady:
            tot = np.array([d[0], abs(d[3]), pe + d[4]])
            if np.all(np.abs((tot - last) / tot) < 1e-3):
                steady = True
            last = tot
        row = [st, P.shape[1], d[0], d[1], d[2], d[3], d[4], pe, 1.0 if steady else 0.0]
        assert np.array_equal(np.array(row), f["hist"][st]), st
    assert np.array_equal(phi, f["phi"])
    assert np.array_equal(P, f["P"])


@pytest.mark.parametrize("case", ["dsmc_steps", "dsmc_sparse"])
def test_dsmc_bitexact(po, case):
    """DSMC_MEX::apply calls of the reference (ch4/Collisions.cpp:108-183),
    replayed with its recorded uniforms: velocities, sigma_cr_max and the
    uniform count reproduced bit for bit.  dsmc_steps: 3000 atoms, three
    calls; dsmc_sparse: 300 atoms in 125 cells (empty, single and two-atom
    cells, whose second pick is redrawn), five calls."""
    f = golden(case)
    g = po.grid(f["grid"], f["x0"], f["xm"])
    P, smax, off = f["P0"], 1e-14, 0
    for st in range(int(f["steps"]) if "steps" in f else 3):
        P, smax, ncol, used, _ = po.dsmc_mex(g, float(f["mass"]), float(f["mpw0"]), float(f["dt"]), f["c"], smax,
                                             P, f["u"][off:])
        off += used
        assert ncol > 0
        assert smax == f["sigma_cr_max"][st], st
    assert off == f["u"].size
    assert np.array_equal(P, f["P"])


def test_neutral_moments_bitexact(po):
    """Species::sampleMoments twice, computeGasProperties and computeMPC of
    the reference (ch4/Species.cpp:191-235) reproduced bit for bit."""
    f = golden("neutral_moments")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    mom = None
    for _ in range(int(f["calls"])):
        mom = po.sample_moments(g, f["P"], mom)
    assert np.array_equal(mom, f["mom"])
    vel, T = po.gas_properties(g, float(f["mass"]), mom)
    assert np.array_equal(vel, f["vel"]) and np.array_equal(T, f["T"])
    assert np.array_equal(po.compute_mpc(g, f["P"]), f["mpc"])


def test_mcc_cex_bitexact(po):
    """Two MCC_CEX::apply calls of the reference (ch4/Collisions.cpp:43-80)
    replayed with its recorded uniforms: velocities and the uniform count
    reproduced bit for bit."""
    f = golden("neutral_mcc")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    P, off = f["P0"], 0
    for _ in range(int(f["steps"])):
        P, ncol, used, _ = po.mcc_cex(g, P, f["den"], f["vel"], float(f["dt"]), f["u"][off:])
        off += used
        assert ncol > 0
    assert off == f["u"].size
    assert np.array_equal(P, f["P"])


def test_ch4_neutral_push_bitexact(po):
    """Five Species::advance(neutrals, neutrals) steps of the reference
    (ch4/Species.cpp:8-100): positions, velocities, per-particle time left,
    removal order and the uniforms of every sphere bounce reproduced bit
    for bit."""
    f = golden("ch4_push")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    sph = f["sphere"]
    P, pdt, off, bounces = f["P0"], f["dt0"], 0, 0
    for _ in range(int(f["steps"])):
        P, pdt, used, _ = po.advance_ch4_neutral(g, tuple(sph[:4]), float(f["mass"]), float(f["dt"]), P, pdt,
                                                 f["u"][off:])
        off += used
        bounces += used // 11
    assert bounces > 50 and off == f["u"].size
    assert np.array_equal(P, f["P"]) and np.array_equal(pdt, f["pdt"])


def test_ch4_ion_push_bitexact(po):
    """Three Species::advance(neutrals, neutrals) steps of an ion species
    (ch4/Species.cpp:8-91, 103-119): E kick, removal at the faces and at the
    sphere, and the neutrals and sputtered atoms the strikes create, with
    their velocities, weights and time left, reproduced bit for bit."""
    f = golden("ch4_ion_push")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    sph, neu = tuple(f["sphere"][:4]), tuple(f["neutral"])
    P, pdt, off = f["P0"], f["dt0"], 0
    N, ndt, sputtered = np.zeros((7, 0)), np.zeros(0), 0
    for _ in range(int(f["steps"])):
        P, pdt, Q, tag, qdt, used = po.advance_ch4_ion(g, f["ef"], sph, float(f["charge"]), float(f["mass"]),
                                                       float(f["mpw0"]), float(f["dt"]), P, pdt, neu, neu,
                                                       f["u"][off:])
        off += used
        N, ndt = np.concatenate([N, Q], axis=1), np.concatenate([ndt, qdt])
        sputtered += int(np.sum(tag == 1))
    assert off == f["u"].size and N.shape[1] > 50 and sputtered > 0
    assert np.array_equal(P, f["P"]) and np.array_equal(pdt, f["pdt"])
    assert np.array_equal(N, f["N"]) and np.array_equal(ndt, f["ndt"])


def test_chemistry_ionize_bitexact(po):
    """ChemistryIonize::apply of the reference (ch4/Collisions.cpp:10-31):
    the ions it adds (at the cell's corner node, as World::pos(int, int, int)
    truncates their sampled positions), their rewound velocities, weights and
    time left (mpw0), and the uniform count, bit for bit."""
    f = golden("ch4_ionize")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    Q, qdt, used = po.chemistry_ionize(g, f["den"], f["rho"], f["ef"], float(f["charge"]), float(f["mass"]),
                                       float(f["mpw0"]), float(f["rate"]), float(f["dt"]), f["u"])
    assert Q.shape[1] > 1000 and used == f["u"].size
    assert np.array_equal(Q, f["P"]) and np.array_equal(qdt, f["pdt"])


def test_ch9mpi_source_bitexact(po):
    """The particle source of the ch9/MPI variant (ch9/MPI/src/Source.cpp:5-72),
    compiled from the reference's sources with a stand-in mpi.h: five calls
    with the remainder carry.  The oracle's restatement (eo_inject_beam, mode
    2 with the remainder count) reproduces counts, remainders, positions and
    rewound velocities bit for bit when fed the same uniforms (the oracle's
    layout reserves a count slot first, unused by the remainder count)."""
    f = golden("inject_ch9mpi")
    g = po.grid([21, 21, 41], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.4])
    ef = po.efield(g, f["phi"])
    rem = np.zeros(1)
    off, out = 0, []
    for c in range(len(f["counts"])):
        k = int(f["used"][c])
        u = np.concatenate([[0.0], f["u"][off:off + k]])
        off += k
        B, used = po.inject_beam(g, ef, QE, 16 * AMU, float(f["dt"]), float(f["spwt"]), float(f["v_drift"]),
                                 float(f["den0"]), float(f["T"]), 2, u, rem=rem)
        assert B.shape[1] == int(f["counts"][c]) and used == k + 1
        assert rem[0] == f["rem"][c]
        out.append(B)
    assert np.array_equal(np.concatenate(out, axis=1), f["P"])
