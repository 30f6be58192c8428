"""DSMC_MEX (ch4/Collisions.h:51-75, ch4/Collisions.cpp:84-183) on the GPU
(espic_dsmc_*), float64 form.

* Replaying the reference's own uniforms (tests/golden/dsmc_steps.npz, three
  apply calls on 3000 atoms in 125 cells), every call draws the same pairs
  and collides the same ones as the oracle: collision counts exact,
  positions and weights exact, velocities within 1e-12 of the largest speed
  (CUDA's pow, cos and sin against the C library's), sigma_cr_max within
  1e-13; after three calls the velocities match the reference's within the
  same bound.
* With the counter-based stream: each collision conserves momentum and
  kinetic energy (1e-12 relative over ten calls), an anisotropic thermal
  spread relaxes towards isotropy, and a second run with the same seed gives
  the same bits.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

AMU = 1.660538921e-27


def test_dsmc_replays_the_reference(espic, po):
    f = golden("dsmc_steps")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    mass, mpw0, dt = float(f["mass"]), float(f["mpw0"]), float(f["dt"])
    with espic.World(*[int(v) for v in f["grid"]], f["x0"], f["xm"]) as w:
        w.setTime(dt, 10)
        s = espic.Species(w, "O", mass, 0.0, mpw0=mpw0, capacity=4096, form=espic.FORM_FP64)
        s.set_particles(f["P0"])
        s.enable_dsmc(c=f["c"], sigma_cr_max=1e-14)
        P, smax, off = f["P0"], 1e-14, 0
        for st in range(3):
            P, smax, ncol, used, coff = po.dsmc_mex(g, mass, mpw0, dt, f["c"], smax, P, f["u"][off:])
            s.dsmc(dt, u=f["u"][off:off + used], cell_off=coff)
            off += used
            got = s.particles()
            smax_g, last, _ = s.dsmc_status()
            assert last == ncol > 0, (st, last, ncol)
            assert abs(smax_g - smax) <= 1e-13 * smax, (st, smax_g, smax)
            assert np.array_equal(got[0:3], P[0:3]) and np.array_equal(got[6], P[6])
            vmax = np.max(np.abs(P[3:6]))
            assert np.max(np.abs(got[3:6] - P[3:6])) <= 1e-12 * vmax, st
        assert abs(smax_g - f["sigma_cr_max"][2]) <= 1e-13 * smax_g
        assert np.max(np.abs(got[3:6] - f["P"][3:6])) <= 1e-12 * np.max(np.abs(f["P"][3:6]))


def gas(n, rng, spread):
    """n atoms uniform in [0, 0.16)^3 drifting at 7 km/s in x with thermal
    spreads `spread` (m/s) per axis"""
    P = np.zeros((7, n))
    P[0:3] = rng.random((3, n)) * 0.16 * 0.999999
    for d in range(3):
        P[3 + d] = spread[d] * rng.standard_normal(n)
    P[3] += 7000.0
    return P


def run_gas(espic, P, mpw0, calls, seed=5, keep=10):
    """`calls` DSMC calls with the counter-based stream; the state after each
    of the first `keep` calls and after the last"""
    with espic.World(17, 17, 17, [0.0, 0.0, 0.0], [0.16, 0.16, 0.16]) as w:
        w.set_seed(seed)
        w.setTime(1e-6, 100)
        s = espic.Species(w, "O", 16 * AMU, 0.0, mpw0=mpw0, capacity=P.shape[1] + 64, form=espic.FORM_FP64)
        P[6] = mpw0
        s.set_particles(P)
        s.enable_dsmc()
        out = []
        for i in range(calls):
            s.dsmc(1e-6)
            if i < keep or i == calls - 1:
                out.append(s.particles())
        return out, s.dsmc_status()


@pytest.fixture(scope="module")
def relaxing(espic):
    rng = np.random.default_rng(11)
    P = gas(200_000, rng, (600.0, 100.0, 100.0))
    states, status = run_gas(espic, P.copy(), 2.5e13, 40)
    return P, states, status


def test_dsmc_conservation_and_relaxation(espic, relaxing):
    P0, states, (smax, last, total) = relaxing
    assert total > P0.shape[1], total  # well over a collision per atom
    assert smax != 1e-14
    v0 = P0[3:6]
    for st in states[:10]:
        v = st[3:6]
        assert np.array_equal(st[0:3], P0[0:3])
        mom0, mom = v0.sum(axis=1), v.sum(axis=1)
        assert np.max(np.abs(mom - mom0)) <= 1e-12 * np.abs(v0).sum()
        e0, e = (v0 * v0).sum(), (v * v).sum()
        assert abs(e - e0) <= 1e-12 * e0
    # thermal spreads about the mean: 36:1 at the start, nearly isotropic after
    def temps(v):
        return ((v - v.mean(axis=1, keepdims=True)) ** 2).mean(axis=1)
    t0, t1 = temps(v0), temps(states[-1][3:6])
    assert t0[0] / t0[1] > 30
    assert t1[0] / t1[1] < 1.3 and t1[0] / t1[2] < 1.3, t1
    assert abs(t1.sum() - t0.sum()) <= 1e-9 * t0.sum()


def test_dsmc_same_seed_same_bits(espic, relaxing):
    P0, states, _ = relaxing
    again, _ = run_gas(espic, P0.copy(), 2.5e13, 3)
    assert np.array_equal(again[-1], states[2])
    other, _ = run_gas(espic, P0.copy(), 2.5e13, 3, seed=6)
    assert not np.array_equal(other[-1], states[2])
