"""The mixed particle form (int32 cell key, float in-cell offset, float
velocity) on the GPU.

* The fused push+deposit (tiles streamed through shared memory, weights of
  equal-cell runs summed in registers) and the separate deposit kernel give
  the same integer charge, bit for bit, on any particle order, count and wall
  kind: the fixed-point sum does not depend on how it is grouped.
* One push against the float64 oracle (ch3/ver2/Species.cpp:7-48 and
  ch2/Species.cpp:7-38): the absorbed count is exact and positions /
  velocities agree to float precision (|dx| <= 1e-5 dh, |dv| <= 1e-5 max|v|).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE, AMU, K = 1.602176565e-19, 1.660538921e-27, 1.380648e-23
SPH = ([33, 33, 65], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.4])
BOX = ([21, 21, 21], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.2])
SPHERE = ([0.0, 0.0, 0.15], 0.05, -100.0)
SPHERE4 = [0.0, 0.0, 0.15, 0.05 * 0.05]
M = 16 * AMU


def state(geo, n, seed, sphere=True, vd=7000.0, vth=800.0):
    rng = np.random.default_rng(seed)
    x0, xm = np.array(geo[1]), np.array(geo[2])
    P = np.zeros((7, n))
    filled = 0
    while filled < n:
        pos = x0 + rng.random((2 * n + 16, 3)) * (xm - x0)
        if sphere:
            c, r = np.array(SPHERE[0]), SPHERE[1]
            pos = pos[np.sum((pos - c) ** 2, axis=1) > r * r]
        k = min(n - filled, pos.shape[0])
        P[0:3, filled:filled + k] = pos[:k].T
        filled += k
    P[3:6] = rng.standard_normal((3, n)) * vth
    P[5] += vd
    P[6] = 40.0
    return P


def smooth_phi(geo):
    ni, nj, nk = geo[0]
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    return (30.0 * np.sin(np.pi * i / (ni - 1)) * np.cos(2.0 * j / nj) * np.sin(3.0 * k / nk)).ravel()


def make(espic, geo, P, walls, sorted_):
    w = espic.World(*geo[0], geo[1], geo[2])
    w.setTime(1e-7 if walls == espic.WALLS_ABSORB else 2e-10, 10)
    if walls == espic.WALLS_ABSORB:
        w.addSphere(*SPHERE)
    w.write(espic.FIELD_PHI, smooth_phi(geo))
    espic.PotentialSolver(w).computeEF()
    s = espic.Species(w, "O+", M, QE, mpw0=40.0, capacity=P.shape[1] + 4096, form=espic.FORM_MIXED,
                      walls=walls)
    s.set_particles(P)
    if sorted_:
        s.sort()
    return w, s


@pytest.mark.parametrize("walls", ["reflect", "absorb"])
@pytest.mark.parametrize("sorted_", [False, True])
@pytest.mark.parametrize("n", [1, 5, 1023, 1024 * 37 + 5, 400_000])
def test_fused_deposit_equals_separate_deposit(espic, walls, sorted_, n):
    wk = espic.WALLS_REFLECT if walls == "reflect" else espic.WALLS_ABSORB
    geo = BOX if walls == "reflect" else SPH
    P = state(geo, n, 3 + n, sphere=walls == "absorb", vd=0.0 if walls == "reflect" else 7000.0,
              vth=8e5 if walls == "reflect" else 800.0)
    w, s = make(espic, geo, P, wk, sorted_)
    with w:
        s.advance(deposit=True)
        fused = s.den
        n_after = s.getNp()
        s.computeNumberDensity()
        sep = s.den
        assert np.array_equal(fused, sep)
        assert n_after == s.particles().shape[1]
        assert np.all(np.isfinite(fused))


@pytest.mark.parametrize("sorted_", [False, True])
def test_mixed_push_sphere_against_oracle(espic, po, sorted_):
    geo = SPH
    n = 300_000
    P = state(geo, n, 5)
    # put a shell of particles just outside the sphere, moving into it
    c, r = np.array(SPHERE[0]), SPHERE[1]
    rng = np.random.default_rng(9)
    d = rng.standard_normal((3, 20000))
    d /= np.linalg.norm(d, axis=0)
    P[0:3, :20000] = c[:, None] + (r + 2e-4) * d
    P[3:6, :20000] = -5e3 * d
    g = po.grid(*geo)
    w, s = make(espic, geo, P, espic.WALLS_ABSORB, sorted_)
    with w:
        start = s.particles()  # the float state the GPU pushes, back in float64
        ef = w.ef
        s.advance(deposit=False)
        got = s.particles()
    want = po.push_sphere(g, ef, SPHERE4, QE, M, 1e-7, start, compact="holes")
    assert got.shape == want.shape  # absorbed count, exact
    dh = np.array(g.dh)
    assert np.max(np.abs(got[0:3] - want[0:3]) / dh[:, None]) <= 1e-5
    assert np.max(np.abs(got[3:6] - want[3:6])) <= 1e-5 * np.max(np.abs(want[3:6]))
    assert got.shape[1] < n  # the shell was absorbed


def test_mixed_push_box_reflect_against_oracle(espic, po):
    geo = BOX
    n = 200_000
    P = state(geo, n, 6, sphere=False, vd=0.0, vth=3e5)
    g = po.grid(*geo)
    w, s = make(espic, geo, P, espic.WALLS_REFLECT, True)
    with w:
        start = s.particles()
        ef = w.ef
        s.advance(deposit=False)
        got = s.particles()
    want = po.push_box(g, ef, QE, M, 2e-10, start)
    dh = np.array(g.dh)
    assert got.shape == want.shape
    assert np.max(np.abs(got[0:3] - want[0:3]) / dh[:, None]) <= 1e-5
    assert np.max(np.abs(got[3:6] - want[3:6])) <= 1e-5 * np.max(np.abs(want[3:6]))


# ---- bit-exact parity of the mixed form with its oracle restatement ------------
# (oracle/espic_oracle.c restates the mixed arithmetic operation by operation:
# float CIC weights, the gather's fused multiply-add chain, the push, the walls,
# the removal order and the 2^-23 fixed-point deposit)

def _ef4(w, po):
    return po.ef_to_f32(w.ef)


def test_to_mixed_matches_oracle(espic, po):
    P = state(SPH, 50_000, 21)
    g = po.grid(*SPH)
    w, s = make(espic, SPH, P, espic.WALLS_ABSORB, False)
    with w:
        cell, off, vel = s.get_mixed()
        back = s.particles()
    c2, o2, v2 = po.to_mixed(g, P)
    assert np.array_equal(cell, c2) and np.array_equal(off, o2) and np.array_equal(vel, v2)
    # and back to float64: x = x0 + (i + f) dh with one fused multiply-add
    assert np.array_equal(back, po.from_mixed(g, c2, o2, v2, 40.0))
    assert np.max(np.abs(back[0:3] - P[0:3]) / np.array(g.dh)[:, None]) <= 2.0 ** -23


@pytest.mark.parametrize("walls", ["reflect", "absorb"])
@pytest.mark.parametrize("n", [1, 777, 300_000])
def test_mixed_push_and_deposit_bitexact(espic, po, walls, n):
    """One fused push + deposit on the GPU against the oracle's mixed
    restatement from the same mixed state: cell keys, offsets, velocities,
    the survivors and their order, and the integer charge (through the
    density) agree bit for bit."""
    wk = espic.WALLS_REFLECT if walls == "reflect" else espic.WALLS_ABSORB
    geo = BOX if walls == "reflect" else SPH
    P = state(geo, n, 40 + n, sphere=walls == "absorb", vd=0.0 if walls == "reflect" else 7000.0,
              vth=8e5 if walls == "reflect" else 800.0)
    if walls == "absorb" and n > 1000:
        c, r = np.array(SPHERE[0]), SPHERE[1]
        d = np.random.default_rng(3).standard_normal((3, 5000))
        d /= np.linalg.norm(d, axis=0)
        P[0:3, :5000] = c[:, None] + (r + 2e-4) * d
        P[3:6, :5000] = -5e3 * d
    g = po.grid(*geo)
    dt = 1e-7 if walls == "absorb" else 2e-10
    w, s = make(espic, geo, P, wk, False)
    with w:
        cell0, off0, vel0 = s.get_mixed()
        ef4 = _ef4(w, po)
        s.advance(deposit=True)
        cell, off, vel = s.get_mixed()
        den = s.den
        vol = w.read(espic.FIELD_NODE_VOL)
    a = po.mix_args(g, QE, M, dt, SPHERE4 if walls == "absorb" else None)
    c2, o2, v2, dead = po.push_mixed(a, ef4, 0 if walls == "reflect" else 1, cell0, off0, vel0)
    assert np.array_equal(cell, c2)
    assert np.array_equal(off, o2) and np.array_equal(vel, v2)
    acc = po.deposit_mixed(g, c2, o2)
    want = po.density_from_fixed(acc, 8388608.0 / 40.0, vol)
    assert np.array_equal(den, want)
    if walls == "absorb" and n > 1000:
        assert dead.sum() > 0


def test_mixed_density_and_potential_against_fp64_oracle(espic, po):
    """The chosen (mixed) form against the float64 oracle on the same
    particles: the ion density within the deposit's quantisation and float
    weight bound (each corner count is off by at most 1/2 of 2^-23 mpw0,
    and the float weight by at most 4 ulps), then phi from the FP32-inner
    Newton-PCG against the oracle's FP64 Newton-PCG on the oracle's density
    (relative 1e-6 of max|phi|, the stated target) and E against the
    oracle's computeEF of that phi (relative 1e-6 of max|E|)."""
    P = state(SPH, 400_000, 77)
    g = po.grid(*SPH)
    w, s = make(espic, SPH, P, espic.WALLS_ABSORB, True)
    with w:
        w.addInlet()
        sol = espic.PotentialSolver(w, espic.SOLVER_PCG, 1000, 1e-4)
        sol.setReferenceValues(0.0, 3.0, 1e10)
        sol.setNewton(nr_max=20, nr_tol=1e-6, pcg_max=20000, pcg_tol=1e-4, fp32_inner=True)
        s.advance(deposit=True)
        den = s.den
        cell, off, vel = s.get_mixed()
        w.computeChargeDensity()
        phi_start = w.phi
        conv = sol.solve()[0]
        phi = w.phi
        sol.computeEF()
        ef = w.ef
        obj = w.object_id
        vol = w.read(espic.FIELD_NODE_VOL)
    assert conv
    # density: the same particles in float64 through the oracle's deposit
    P64 = po.from_mixed(g, cell, off, vel, 40.0)
    den64 = po.divide_volume(po.deposit_fp64(g, P64), vol)
    count = po.deposit_fp64(g, np.vstack([P64[:6], np.ones((1, P64.shape[1]))]))
    contrib = np.ceil(count * 8 + 8)  # corner contributions per node, generous
    bound = contrib * 40.0 * 5 * 2.0 ** -24 / np.where(vol > 0, vol, 1)
    assert np.all(np.abs(den - den64) <= bound)
    # RMS error against the RMS density (nodes grazed by one corner weight
    # carry relative errors up to the quantum over a tiny density)
    assert np.sqrt(np.mean((den - den64) ** 2)) <= 1e-6 * np.sqrt(np.mean(den64 ** 2))
    # phi: the oracle's float64 Newton-PCG on the oracle's charge density
    rho64 = den64 * QE
    phi64, conv64, _, _ = po.newton_pcg(g, phi_start, rho64, obj, 0.0, 3.0, 1e10, 30, 1e-10, 20000, 1e-12)
    assert conv64
    assert np.max(np.abs(phi - phi64)) <= 1e-6 * np.max(np.abs(phi64))
    ef64 = po.efield(g, phi64)
    assert np.max(np.abs(ef - ef64)) <= 1e-6 * np.max(np.abs(ef64))


@pytest.mark.parametrize("walls", ["reflect", "absorb"])
def test_tile_segment_push_matches_oracle_over_steps(espic, po, walls):
    """After a sort the push runs over tile segments (one block per 8^3-cell
    tile, E and the deposit staged in shared-memory boxes), particles
    appended since the sort by a tail kernel, and particles that the removal
    moved into a segment through the global fallback.  Six steps with
    particles appended before each: every step's cell keys, offsets,
    velocities, survivors and integer charge equal the oracle's mixed
    restatement run on the GPU's state, bit for bit."""
    wk = espic.WALLS_REFLECT if walls == "reflect" else espic.WALLS_ABSORB
    geo = BOX if walls == "reflect" else SPH
    dt = 1e-7 if walls == "absorb" else 2e-10
    P = state(geo, 200_000, 61, sphere=walls == "absorb", vd=0.0 if walls == "reflect" else 7000.0,
              vth=8e5 if walls == "reflect" else 800.0)
    g = po.grid(*geo)
    rng = np.random.default_rng(62)
    w, s = make(espic, geo, P, wk, True)
    with w:
        ef4 = _ef4(w, po)
        vol = w.read(espic.FIELD_NODE_VOL)
        a = po.mix_args(g, QE, M, dt, SPHERE4 if walls == "absorb" else None)
        dead_total = 0
        for st in range(6):
            x0, xm = np.array(geo[1]), np.array(geo[2])
            pos = x0 + (0.05 + 0.9 * rng.random((500, 3))) * (xm - x0)
            if walls == "absorb":
                pos = pos[np.sum((pos - np.array(SPHERE[0])) ** 2, axis=1) > SPHERE[1] ** 2]
            vel = rng.standard_normal(pos.shape) * (8e5 if walls == "reflect" else 800.0)
            s.addParticles(pos, vel)
            cell0, off0, vel0 = s.get_mixed()
            s.advance(deposit=True)
            cell, off, vv = s.get_mixed()
            den = s.den
            c2, o2, v2, dead = po.push_mixed(a, ef4, 0 if walls == "reflect" else 1, cell0, off0, vel0)
            assert np.array_equal(cell, c2), st
            assert np.array_equal(off, o2) and np.array_equal(vv, v2), st
            want = po.density_from_fixed(po.deposit_mixed(g, c2, o2), 8388608.0 / 40.0, vol)
            assert np.array_equal(den, want), st
            dead_total += int(dead.sum())
        if walls == "absorb":
            assert dead_total > 0


def test_tile_deposit_with_appended_ions(espic):
    """computeNumberDensity of a tile-sorted species whose ions were pushed
    and then joined by injected ions (the tile segments plus the appended
    tail): the same integer charge as the per-ion deposit of the same ions
    in a species that was never sorted"""
    geo = SPH
    P = state(geo, 200_000, 11)
    w, s = make(espic, geo, P, espic.WALLS_ABSORB, True)
    with w:
        # n v A dt / mpw0 = 4e9 * 7000 * 0.04 * 1e-7 / 40 = 2800 ions a
        # sample, within the 4096 spare slots
        src = espic.BeamSource(s, 7000.0, 4e9)
        s.advance(deposit=False)
        n_pushed = s.getNp()
        src.sample()
        cell, off, vel = s.get_mixed()
        assert cell.size > n_pushed + 2000  # the injected tail is there
        s.computeNumberDensity()
        tiled = s.den
    w2, s2 = make(espic, geo, P, espic.WALLS_ABSORB, False)
    with w2:
        s2.set_mixed(cell, off, vel)
        s2.computeNumberDensity()
        plain = s2.den
    assert np.array_equal(tiled, plain)
    assert np.sum(tiled) > 0
