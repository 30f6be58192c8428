"""ch4 neutral-species kernels on the GPU (float64 form), through the C-ABI.

* Species::sampleMoments / computeGasProperties / computeMPC
  (ch4/Species.cpp:191-235) against the reference's own outputs
  (tests/golden/neutral_moments.npz; the oracle reproduces them bit for bit):
  the sampled sums within 1e-12 of each sum's largest node value (64-bit
  fixed-point products, summed exactly, against float64 sums in particle
  order), the stream velocity within 1e-10 of its largest component, the
  temperature within 1e-6 of its largest value (T subtracts two terms about
  150x larger than itself at this drift), macroparticles per cell exact;
  a species of uniform weight (no stored weight row) against the oracle.
* MCC_CEX::apply (ch4/Collisions.cpp:43-80) replaying the reference's
  uniforms (tests/golden/neutral_mcc.npz, two calls on 2000 ions): the same
  particles collide and the velocities match bit for bit.
* With the counter-based stream: the collision count of 200k ions lies
  within 5 standard deviations of the sum of their probabilities, and the
  same seed gives the same bits.
"""
import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

AMU, QE = 1.660538921e-27, 1.602176565e-19


def world_of(espic, f):
    return espic.World(*[int(v) for v in f["grid"]], f["x0"], f["xm"])


def test_moments_gas_properties_mpc(espic):
    f = golden("neutral_moments")
    nn = int(np.prod(f["grid"]))
    with world_of(espic, f) as w:
        w.setTime(1e-7, 10)
        s = espic.Species(w, "O", float(f["mass"]), 0.0, mpw0=1e12, capacity=4096, form=espic.FORM_FP64,
                          weight_bound=2e12)
        s.set_particles(f["P"])
        for _ in range(int(f["calls"])):
            s.sampleMoments()
        mom = s.moments
        ref = f["mom"].reshape(7, nn)
        for q in range(7):
            assert np.max(np.abs(mom[q] - ref[q])) <= 1e-12 * np.max(np.abs(ref[q])), q
        s.computeGasProperties()
        vel, T = s.vel, s.T
        rv = f["vel"].reshape(nn, 3)
        assert np.max(np.abs(vel - rv)) <= 1e-10 * np.max(np.abs(rv))
        assert np.array_equal(T == 0, f["T"] == 0)
        assert np.max(np.abs(T - f["T"])) <= 1e-6 * np.max(f["T"])
        s.computeMPC()
        assert np.array_equal(s.mpc, f["mpc"])
        # clearSamples then one call: half of the two-call sums
        s.clearSamples()
        assert not np.any(s.moments)
        s.sampleMoments()
        one = s.moments
        for q in range(7):
            assert np.max(np.abs(2 * one[q] - ref[q])) <= 1e-12 * np.max(np.abs(ref[q])), q


def test_moments_uniform_weights(espic, po):
    """A species whose particles all carry mpw0 stores no weight row: the
    moments take mpw0 (checked against the oracle on the same atoms)."""
    f = golden("neutral_moments")
    nn = int(np.prod(f["grid"]))
    P = f["P"].copy()
    P[6] = 1e12
    g = po.grid(f["grid"], f["x0"], f["xm"])
    ref = po.sample_moments(g, P).reshape(7, nn)
    with world_of(espic, f) as w:
        w.setTime(1e-7, 10)
        s = espic.Species(w, "O", float(f["mass"]), 0.0, mpw0=1e12, capacity=4096, form=espic.FORM_FP64)
        s.set_particles(P)
        s.sampleMoments()
        mom = s.moments
        for q in range(7):
            assert np.max(np.abs(mom[q] - ref[q])) <= 1e-12 * np.max(np.abs(ref[q])), q


def mcc_world(espic, f, ions):
    w = world_of(espic, f)
    w.setTime(float(f["dt"]), 10)
    src = espic.Species(w, "O+", 16 * AMU, QE, mpw0=5e2, capacity=ions.shape[1] + 64, form=espic.FORM_FP64)
    tgt = espic.Species(w, "O", 16 * AMU, 0.0, mpw0=1e12, capacity=64, form=espic.FORM_FP64)
    src.set_particles(ions)
    w.write(espic.FIELD_DEN, f["den"], sp=tgt.id)
    w.write(espic.FIELD_VEL, f["vel"], sp=tgt.id)
    return w, src, tgt


def test_mcc_replays_the_reference(espic, po):
    f = golden("neutral_mcc")
    g = po.grid(f["grid"], f["x0"], f["xm"])
    w, src, tgt = mcc_world(espic, f, f["P0"])
    with w:
        mcc = espic.MCC_CEX(src, tgt, w)
        P, off = f["P0"], 0
        for st in range(int(f["steps"])):
            P, ncol, used, poff = po.mcc_cex(g, P, f["den"], f["vel"], float(f["dt"]), f["u"][off:])
            got_n = mcc.apply(float(f["dt"]), u=f["u"][off:off + used], p_off=poff)
            off += used
            assert got_n == ncol > 0, (st, got_n, ncol)
            assert np.array_equal(src.particles(), P), st
        assert np.array_equal(src.particles(), f["P"])


def test_mcc_counter_stream(espic):
    f = golden("neutral_mcc")
    rng = np.random.default_rng(9)
    n = 200_000
    ions = np.zeros((7, n))
    ions[0:3] = rng.random((3, n)) * 0.05 * 0.999999
    ions[3:6] = 2000 * rng.standard_normal((3, n))
    ions[6] = 5e2
    dt = float(f["dt"])
    # each ion's probability 1 - exp(-n sigma |v - v_t| dt) from the
    # trilinearly gathered target fields
    nn = int(np.prod(f["grid"]))
    lc = (ions[0:3].T - np.array(f["x0"])) / ((np.array(f["xm"]) - np.array(f["x0"])) / (np.array(f["grid"]) - 1))
    i = np.minimum(lc.astype(int), np.array(f["grid"]) - 2)
    d = lc - i
    ni, nj = int(f["grid"][0]), int(f["grid"][1])
    den, vel = f["den"], f["vel"].reshape(nn, 3)
    nd, vt = np.zeros(n), np.zeros((n, 3))
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                wgt = (d[:, 0] if a else 1 - d[:, 0]) * (d[:, 1] if b else 1 - d[:, 1]) * (d[:, 2] if c else 1 - d[:, 2])
                node = ((i[:, 2] + c) * nj + i[:, 1] + b) * ni + i[:, 0] + a
                nd += wgt * den[node]
                vt += wgt[:, None] * vel[node]
    pc = 1 - np.exp(-nd * 1e-16 * np.linalg.norm(ions[3:6].T - vt, axis=1) * dt)

    def run(seed):
        w, src, tgt = mcc_world(espic, f, ions)
        with w:
            w.set_seed(seed)
            k = espic.MCC_CEX(src, tgt, w).apply(dt, count=True)
            return k, src.particles()

    k, P = run(3)
    mu, sd = pc.sum(), np.sqrt((pc * (1 - pc)).sum())
    assert abs(k - mu) < 5 * sd, (k, mu, sd)
    stopped = np.all(P[3:6] == 0, axis=0)
    assert stopped.sum() == k
    assert np.array_equal(P[:, ~stopped], ions[:, ~stopped])
    k2, P2 = run(3)
    assert k2 == k and np.array_equal(P2, P)
    k3, P3 = run(4)
    assert not np.array_equal(P3, P)


def test_moments_need_the_float64_form(espic):
    with espic.World(5, 5, 5, [0, 0, 0], [0.04, 0.04, 0.04]) as w:
        s = espic.Species(w, "O+", 16 * AMU, QE, mpw0=1.0, capacity=64, form=espic.FORM_MIXED)
        with pytest.raises(espic.EspicError):
            s.sampleMoments()
