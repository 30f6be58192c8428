"""The oracle's restatement of the mixed particle form (int32 cell, float
offsets and velocities, 2^-23 fixed-point deposit) against the float64
oracle, which is pinned bit for bit to the reference (test_oracle_golden.py).
CPU only: this bounds how far the chosen form may sit from the reference's
arithmetic, before any GPU run compares the GPU with the restatement.

* float64 -> mixed -> float64 moves a particle by at most 2^-24 of a cell;
* the mixed deposit's density lies within its quantisation bound of the
  float64 oracle's density of the same particles (the golden box particles
  of tests/golden/box_deposit.npz, on which the float64 deposit reproduces
  the reference's);
* one mixed push stays within float precision of the float64 push
  (ch3/ver2/Species.cpp:7-48) and absorbs the same particles, away from
  ties at the sphere and the faces."""
import numpy as np

from conftest import golden

QE, AMU = 1.602176565e-19, 1.660538921e-27
M = 16 * AMU
BOX = ([21, 21, 21], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.2])  # the grid of box_deposit.npz


def test_mixed_roundtrip(po):
    f = golden("box_deposit")
    g = po.grid(*BOX)
    P = f["Pi"]
    cell, off, vel = po.to_mixed(g, P)
    back = po.from_mixed(g, cell, off, vel, 1.0)
    dh = np.array(g.dh)[:, None]
    assert np.max(np.abs(back[0:3] - P[0:3]) / dh) <= 2.0 ** -24 * 1.01
    assert np.array_equal(back[3:6], P[3:6].astype(np.float32).astype(np.float64))
    c2, o2, v2 = po.to_mixed(g, back)
    assert np.array_equal(c2, cell) and np.array_equal(o2, off) and np.array_equal(v2, vel)


def test_mixed_deposit_within_bound_of_reference_density(po):
    f = golden("box_deposit")
    g = po.grid(*BOX)
    vol = po.node_volumes(g)
    P = f["Pi"].copy()
    mpw0 = float(P[6, 0])
    P[6] = mpw0  # the mixed form carries one weight per species
    cell, off, vel = po.to_mixed(g, P)
    acc = po.deposit_mixed(g, cell, off)
    den_mixed = po.density_from_fixed(acc, 8388608.0 / mpw0, vol)
    den64 = po.divide_volume(po.deposit_fp64(g, po.from_mixed(g, cell, off, vel, mpw0)), vol)
    ones = po.deposit_fp64(g, po.from_mixed(g, cell, off, vel, 1.0))
    bound = (np.ceil(ones) + 8) * 8 * mpw0 * 5 * 2.0 ** -24 / vol
    assert np.all(np.abs(den_mixed - den64) <= bound)
    assert np.max(np.abs(den_mixed - den64)) <= 1e-6 * np.max(den64)


def test_mixed_push_close_to_float64_push(po):
    rng = np.random.default_rng(5)
    g = po.grid([33, 33, 65], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.4])
    n = 100_000
    x0, xm = np.array(g.x0), np.array(g.xm)
    P = np.zeros((7, n))
    P[0:3] = x0[:, None] + rng.random((3, n)) * (xm - x0)[:, None]
    P[3:6] = rng.standard_normal((3, n)) * 800.0
    P[5] += 7000.0
    P[6] = 40.0
    sphere = [0.0, 0.0, 0.15, 0.05 * 0.05]
    out = np.sum((P[0:3] - np.array(sphere[:3])[:, None]) ** 2, axis=0) > sphere[3]
    P = np.ascontiguousarray(P[:, out])
    ni, nj, nk = 33, 33, 65
    k, j, i = np.meshgrid(np.arange(nk), np.arange(nj), np.arange(ni), indexing="ij")
    phi = (30.0 * np.sin(np.pi * i / (ni - 1)) * np.cos(2.0 * j / nj) * np.sin(3.0 * k / nk)).ravel()
    ef = po.efield(g, phi)
    cell, off, vel = po.to_mixed(g, P)
    P0 = po.from_mixed(g, cell, off, vel, 40.0)
    a = po.mix_args(g, QE, M, 1e-7, sphere)
    c2, o2, v2, dead = po.push_mixed(a, po.ef_to_f32(ef), 1, cell, off, vel, compact=False)
    want = po.push_sphere(g, ef, sphere, QE, M, 1e-7, P0, compact=None)
    dead64 = ~(want[6] > 0)
    # particles whose fate is a tie within float precision are left out
    got = po.from_mixed(g, c2, o2, v2, 40.0)
    keep = ~dead64 & (dead == 0)
    assert np.mean((dead == 1) != dead64) < 1e-3
    dh = np.array(g.dh)[:, None]
    assert np.max(np.abs(got[0:3, keep] - want[0:3, keep]) / dh) <= 1e-5
    assert np.max(np.abs(got[3:6, keep] - want[3:6, keep])) <= 1e-5 * np.max(np.abs(want[3:6, keep]))
