"""The ch4 neutral push on the GPU (espic_advance_ch4; Species::advance of a
species of charge 0 with the sphere's diffuse reflection,
ch4/Species.cpp:8-100), float64 form.

* Replaying the reference's uniforms (tests/golden/ch4_push.npz, five steps
  of 3000 atoms, ~120 bounces): each step is checked against the oracle run
  on the GPU's own state (the oracle removes the dead in the GPU's order):
  the same bounces, the same survivors in the same order, positions and
  velocities within 1e-12 of each row's largest value (CUDA's cos and sin
  against the C library's in the re-emitted velocities).
* Time per particle: particles appended since the last push (set, added)
  move for two steps' time, the others for one (a source's addParticle
  leaves a particle one dt, ch4/Species.h:65, and advance adds one).
* Counter-based stream: same seed, same bits; a charged species is refused.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

AMU, QE = 1.660538921e-27, 1.602176565e-19


def ch4_world(espic, f, sphere=True):
    w = espic.World(*[int(v) for v in f["grid"]], f["x0"], f["xm"])
    w.setTime(float(f["dt"]), 100)
    if sphere:
        sph = f["sphere"]
        w.addSphere(sph[:3], float(sph[3]), float(sph[4]))
    s = espic.Species(w, "O", float(f["mass"]), 0.0, mpw0=1e12, capacity=4096, form=espic.FORM_FP64)
    return w, s


def test_ch4_push_replays_the_reference(espic, po):
    f = golden("ch4_push")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    sph = tuple(f["sphere"][:4])
    mass, dt = float(f["mass"]), float(f["dt"])
    w, s = ch4_world(espic, f)
    with w:
        s.set_particles(f["P0"])
        P, pdt, off, total = f["P0"], f["dt0"], 0, 0
        for st in range(int(f["steps"])):
            u = f["u"][off:]
            want, want_pdt, used, p_off = po.advance_ch4_neutral(g, sph, mass, dt, P, pdt, u, holes=True)
            b = s.advance_ch4(pdt=pdt, u=u[:used], p_off=p_off)
            got = s.particles()
            # positions and velocities first: a mismatch there says whether
            # the particles moved at all before the bounce count is judged
            assert got.shape == want.shape, (st, got.shape, want.shape)
            for r in range(7):
                scale = max(np.max(np.abs(want[r])), 1e-300)
                assert np.max(np.abs(got[r] - want[r])) <= 1e-12 * scale, (st, r)
            assert 11 * b == used, (st, b, used)
            off += used
            total += b
            P, pdt = got, want_pdt
        assert total > 50


def test_ch4_push_time_of_new_particles(espic):
    f = golden("ch4_push")
    dt = float(f["dt"])
    rng = np.random.default_rng(3)
    n = 64
    P = np.zeros((7, n))
    P[0] = -0.05 + 0.1 * rng.random(n)
    P[1] = -0.05 + 0.1 * rng.random(n)
    P[2] = 0.30 + 0.05 * rng.random(n)
    P[3:6] = rng.standard_normal((3, n))
    P[6] = 1e12
    w, s = ch4_world(espic, f, sphere=False)
    with w:
        s.set_particles(P)
        assert s.advance_ch4(count=True) == 0
        x1 = s.particles()
        assert np.array_equal(x1[0:3], P[0:3] + P[3:6] * (dt + dt))
        s.advance_ch4()
        x2 = s.particles()
        assert np.array_equal(x2[0:3], x1[0:3] + x1[3:6] * dt)
        # appended particles: two steps' time; the others one
        s.addParticles(P[0:3, :8].T.copy(), P[3:6, :8].T.copy())
        s.advance_ch4()
        x3 = s.particles()
        assert x3.shape[1] == n + 8
        assert np.array_equal(x3[0:3, :n], x2[0:3] + x2[3:6] * dt)
        assert np.array_equal(x3[0:3, n:], P[0:3, :8] + P[3:6, :8] * (dt + dt))


def test_ch4_push_counter_stream(espic):
    f = golden("ch4_push")

    def run(seed):
        w, s = ch4_world(espic, f)
        with w:
            w.set_seed(seed)
            s.set_particles(f["P0"])
            b = [s.advance_ch4(count=True) for _ in range(3)]
            return b, s.particles()

    b, P = run(8)
    assert sum(b) > 20
    assert P.shape[1] < f["P0"].shape[1]  # atoms leave through the far face
    b2, P2 = run(8)
    assert b2 == b and np.array_equal(P2, P)
    _, P3 = run(9)
    assert not (P3.shape == P.shape and np.array_equal(P3, P))


def test_ch4_push_refuses_charged_species(espic):
    f = golden("ch4_push")
    w = espic.World(*[int(v) for v in f["grid"]], f["x0"], f["xm"])
    with w:
        w.setTime(float(f["dt"]), 10)
        s = espic.Species(w, "O+", 16 * AMU, QE, mpw0=1.0, capacity=64, form=espic.FORM_FP64)
        with pytest.raises(espic.EspicError):
            s.advance_ch4()
