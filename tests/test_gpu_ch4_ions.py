"""ch4's ion branch and ionization on the GPU, float64 form:
espic_advance_ch4_ions (Species::advance(neutrals, spherium) of a charged
species, ch4/Species.cpp:8-91) and espic_chemistry_ionize
(ChemistryIonize::apply, ch4/Collisions.cpp:10-31).

* Replaying the reference's uniforms (tests/golden/ch4_ion_push.npz: three
  steps of 1500 O+ in a given E field, ~70 particles created): each step is
  checked against the oracle run on the GPU's own state (the oracle removes
  the dead in the GPU's order).  Surviving ions and the strike points are
  bit-exact (no transcendental on their path); created velocities go
  through CUDA's cos and sin in the diffuse direction, so they are held to
  1e-12 of each row's largest value.
* Separate neutral and spherium targets: each receives its own particles in
  ion order.
* Ionization replaying the reference's uniforms (tests/golden/ch4_ionize.npz,
  2408 ions over 2000 cells): positions, rewound velocities and weights
  bit-exact.
* Counter-based streams: same seed, same particles; the mean count of the
  ionization within 5 sigma of its expectation.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

AMU, QE = 1.660538921e-27, 1.602176565e-19


def ion_world(espic, f, spherium_mpw0=None):
    w = espic.World(*[int(v) for v in f["grid"]], f["x0"], f["xm"])
    w.setTime(float(f["dt"]), 100)
    sph = f["sphere"]
    w.addSphere(sph[:3], float(sph[3]), float(sph[4]))
    ions = espic.Species(w, "O+", float(f["mass"]), float(f["charge"]), mpw0=float(f["mpw0"]), capacity=4096,
                         form=espic.FORM_FP64)
    neu_mpw0, neu_q, neu_m = (float(v) for v in f["neutral"])
    neu = espic.Species(w, "O", neu_m, neu_q, mpw0=neu_mpw0, capacity=4096, form=espic.FORM_FP64)
    sph_sp = None
    if spherium_mpw0 is not None:
        sph_sp = espic.Species(w, "Sph", 100 * AMU, 0.0, mpw0=spherium_mpw0, capacity=4096, form=espic.FORM_FP64)
    w.write(espic.FIELD_EF, np.asarray(f["ef"], dtype=np.float64))
    return w, ions, neu, sph_sp


def close_rows(got, want, rows, what):
    assert got.shape == want.shape, (what, got.shape, want.shape)
    for r in rows:
        scale = max(np.max(np.abs(want[r])), 1e-300) if want.shape[1] else 1.0
        assert np.max(np.abs(got[r] - want[r]), initial=0.0) <= 1e-12 * scale, (what, r)


def by_position(P):
    return P[:, np.lexsort((P[2], P[1], P[0]))]


def test_ch4_ion_push_replays_the_reference(espic, po):
    f = golden("ch4_ion_push")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    sph, neu_t = tuple(f["sphere"][:4]), tuple(f["neutral"])
    q, m, mpw0, dt = float(f["charge"]), float(f["mass"]), float(f["mpw0"]), float(f["dt"])
    w, ions, neu, _ = ion_world(espic, f)
    with w:
        ions.set_particles(f["P0"])
        P, pdt, off, created, strikes = f["P0"], f["dt0"], 0, 0, 0
        for st in range(int(f["steps"])):
            u = f["u"][off:]
            want, want_pdt, Q, tag, qdt, used, p_off = po.advance_ch4_ion_holes(g, f["ef"], sph, q, m, mpw0, dt, P,
                                                                                 pdt, neu_t, neu_t, u)
            b = ions.advance_ch4_ions(neu, pdt=pdt, u=u[:used], p_off=p_off)
            got = ions.particles()
            assert got.shape == want.shape, (st, got.shape, want.shape)
            assert np.array_equal(got[:6], want[:6]), st
            N = neu.particles()
            assert N.shape[1] == created + Q.shape[1], st
            new = N[:, created:]
            assert np.array_equal(new[0:3], Q[0:3]), st  # strike points
            close_rows(new, Q, range(3, 7), ("created", st))
            # two count uniforms per strike and 11 per created particle
            assert used == 2 * b + 11 * Q.shape[1], (st, b, used, Q.shape)
            if st == 0:
                # the first step starts from the reference's own ion order:
                # its created particles are the reference's first ones
                k = Q.shape[1]
                assert np.array_equal(new[0:3], f["N"][0:3, :k])
                close_rows(new, f["N"][:, :k], range(3, 7), "reference step 1")
            off += used
            created += Q.shape[1]
            strikes += b
            P, pdt = got, want_pdt
        assert off == f["u"].size
        # the reference's own run: the same surviving ions (its swap-with-last
        # removal orders them differently; from the second step on it also
        # hands the uniforms to the ions in that other order, so only the
        # first step's created particles are comparable one to one)
        assert np.array_equal(by_position(ions.particles())[:6], by_position(f["P"])[:6])
        assert strikes > 20 and created > 50


def test_ch4_ion_push_separate_spherium(espic, po):
    f = golden("ch4_ion_push")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    sph, neu_t = tuple(f["sphere"][:4]), tuple(f["neutral"])
    q, m, mpw0, dt = float(f["charge"]), float(f["mass"]), float(f["mpw0"]), float(f["dt"])
    sph_mpw0 = 4e10  # 0.1 * 2e11 / 4e10 = 0.5 sputtered atoms per fast strike
    w, ions, neu, spc = ion_world(espic, f, spherium_mpw0=sph_mpw0)
    with w:
        ions.set_particles(f["P0"])
        u = np.random.default_rng(5).random(20000)
        sph_t = (sph_mpw0, 0.0, 100 * AMU)
        want, _, Q, tag, _, used, p_off = po.advance_ch4_ion_holes(g, f["ef"], sph, q, m, mpw0, dt, f["P0"],
                                                                  f["dt0"], neu_t, sph_t, u)
        b = ions.advance_ch4_ions(neu, spc, pdt=f["dt0"], u=u[:used], p_off=p_off)
        assert b > 10 and np.sum(tag == 1) > 2
        assert np.array_equal(ions.particles()[:6], want[:6])
        for sp, t in ((neu, 0), (spc, 1)):
            got, exp = sp.particles(), Q[:, tag == t]
            assert np.array_equal(got[0:3], exp[0:3]), t
            close_rows(got, exp, range(3, 7), ("target", t))


def test_ch4_ion_push_counter_stream(espic):
    f = golden("ch4_ion_push")

    def run(seed):
        w, ions, neu, _ = ion_world(espic, f)
        with w:
            w.set_seed(seed)
            ions.set_particles(f["P0"])
            b = [ions.advance_ch4_ions(neu) for _ in range(3)]
            return b, ions.particles(), neu.particles()

    b, P, N = run(8)
    assert sum(b) > 20 and N.shape[1] >= 2 * sum(b) - 5  # mpw0 ratio 2: two neutrals per strike
    b2, P2, N2 = run(8)
    assert b2 == b and np.array_equal(P2, P) and np.array_equal(N2, N)
    _, _, N3 = run(9)
    assert not (N3.shape == N.shape and np.array_equal(N3, N))


def test_ch4_ion_push_refusals(espic):
    f = golden("ch4_ion_push")
    w, ions, neu, _ = ion_world(espic, f)
    with w:
        with pytest.raises(espic.EspicError):
            neu.advance_ch4_ions(ions)  # a neutral species
        with pytest.raises(espic.EspicError):
            ions.advance_ch4_ions(ions)  # its own target
        with pytest.raises(espic.EspicError):
            ions.advance_ch4()  # the neutral push


def ionize_world(espic, f):
    w = espic.World(*[int(v) for v in f["grid"]], f["x0"], f["xm"])
    w.setTime(float(f["dt"]), 100)
    neu = espic.Species(w, "O", float(f["mass"]), 0.0, mpw0=1e12, capacity=64, form=espic.FORM_FP64)
    ions = espic.Species(w, "O+", float(f["mass"]), float(f["charge"]), mpw0=float(f["mpw0"]), capacity=8192,
                         form=espic.FORM_FP64)
    w.write(espic.FIELD_DEN, np.asarray(f["den"], dtype=np.float64), sp=neu.id)
    w.write(espic.FIELD_RHO, np.asarray(f["rho"], dtype=np.float64))
    w.write(espic.FIELD_EF, np.asarray(f["ef"], dtype=np.float64))
    return w, neu, ions


def test_chemistry_ionize_replays_the_reference(espic, po):
    f = golden("ch4_ionize")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    Q, _, used, cell_off = po.chemistry_ionize_offsets(g, f["den"], f["rho"], f["ef"], float(f["charge"]),
                                                       float(f["mass"]), float(f["mpw0"]), float(f["rate"]),
                                                       float(f["dt"]), f["u"])
    assert np.array_equal(Q, f["P"])
    w, neu, ions = ionize_world(espic, f)
    with w:
        chem = espic.ChemistryIonize(neu, ions, w, float(f["rate"]))
        n = chem.apply(float(f["dt"]), u=f["u"][:used], cell_off=cell_off)
        assert n == Q.shape[1] > 1000
        got = ions.particles()
        assert np.array_equal(got, Q)


def test_chemistry_ionize_counter_stream(espic):
    f = golden("ch4_ionize")
    ni, nj, nk = (int(v) for v in f["grid"])
    x0, xm = np.asarray(f["x0"]), np.asarray(f["xm"])
    dh = (xm - x0) / (np.array([ni, nj, nk]) - 1)
    # at the cell centre every corner weighs 1/8: y = rate n_a n_e dt dV / mpw0
    # per cell; a cell adds floor(y + U), of mean y and variance frac(y)(1 - frac(y))
    def centre(a):
        a = np.asarray(a).reshape(nk, nj, ni)
        return 0.125 * sum(a[k:nk - 1 + k, j:nj - 1 + j, i:ni - 1 + i] for i in (0, 1) for j in (0, 1) for k in (0, 1))
    y = (float(f["rate"]) * centre(f["den"]) * centre(f["rho"]) / QE * float(f["dt"]) * np.prod(dh)
         / float(f["mpw0"]))
    fr = y - np.floor(y)
    mean, sd = float(y.sum()), float(np.sqrt(np.sum(fr * (1 - fr))))
    counts = []
    for seed in (3, 3, 4):
        w, neu, ions = ionize_world(espic, f)
        with w:
            w.set_seed(seed)
            chem = espic.ChemistryIonize(neu, ions, w, float(f["rate"]))
            counts.append((chem.apply(float(f["dt"])), ions.particles()))
    (n0, P0), (n1, P1), (n2, P2) = counts
    assert n0 == n1 and np.array_equal(P0, P1)
    assert not (n2 == n0 and np.array_equal(P2, P0))
    for n in (n0, n2):
        assert abs(n - mean) < 5 * sd + 1, (n, mean, sd)
    assert np.all(P0[6] == float(f["mpw0"]))
