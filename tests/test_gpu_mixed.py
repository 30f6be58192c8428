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
