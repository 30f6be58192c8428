"""CPU check of the float-estimated division that the multigrid sweeps, the
restrictions and the E kernel use for node coordinates (div_small in
csrc/espic_world.h): for n < 2^24, trunc(float(n) * RN(1/d)) is within one of
n // d, so one remainder test makes it exact.  Emulated with numpy float32,
whose products round to nearest like the device's float multiply."""
import numpy as np


def div_small(n, d):
    inv = np.float32(1.0) / np.float32(d)
    q = np.trunc(n.astype(np.float32) * inv).astype(np.int64)
    est = q.copy()
    r = n - q * d
    q = np.where(r < 0, q - 1, np.where(r >= d, q + 1, q))
    return est, q


def test_float_estimated_division_is_exact_below_2_pow_24():
    rng = np.random.default_rng(24)
    top = 1 << 24
    for d in range(1, 4097):
        # every remainder class near multiples of d across the range, plus
        # random samples and the last representable values
        k = rng.integers(0, top // d, 256)
        n = np.concatenate([k * d, k * d + d - 1, rng.integers(0, top, 256),
                            np.arange(top - 64, top)]).astype(np.int64)
        n = n[(n >= 0) & (n < top)]
        est, q = div_small(n, d)
        want = n // d
        assert np.all(np.abs(est - want) <= 1), d
        assert np.array_equal(q, want), d


def dsmc_axis(x0, xm, dh, nc):
    """host side of the DSMC cell estimate (dsmc_axis in csrc/k_fp64.cu)"""
    L = max(abs(x0), abs(xm)) + dh
    err = 3.01 * 2.0 ** -24 * (nc + 1.0) + (2.0 ** -23 * L + 2.0 ** -24 * abs(x0)) / dh
    tol = 2 * err + 1e-12
    return np.float32(x0), np.float32(1.0 / dh), np.float32(tol if tol < 0.01 else 2.0), nc


def dsmc_coord(x, x0, dh, ax):
    """device side (dsmc_coord): x cut to 24 leading bits by integer
    operations, q = (x_f - x0_f) * (1/dh)_f in float, accepted when q lies
    farther than tol from an integer, else the float64 division"""
    x0f, invf, tol, nc = ax
    bits = x.view(np.uint64)
    hi = (bits >> np.uint64(32)).astype(np.uint32)
    lo = (bits & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    fe = ((hi >> 20) & 0x7FF).astype(np.int64) - 896
    fb = (hi & 0x80000000) | (np.clip(fe, 0, 255).astype(np.uint32) << 23) | ((hi & 0xFFFFF) << 3) | (lo >> 29)
    xf = np.where(fe >= 1, fb.astype(np.uint32).view(np.float32), np.float32(0))
    q = ((xf - x0f).astype(np.float32) * invf).astype(np.float32)
    k = np.trunc(q).astype(np.int64)
    fr = (q - k.astype(np.float32)).astype(np.float32)
    fast = (fe <= 254) & (q >= 0) & (q < np.float32(nc)) & (fr > tol) & (fr < np.float32(1) - tol)
    exact = np.trunc((x - x0) / dh).astype(np.int64)
    return np.where(fast, k, exact), exact, fast


def test_dsmc_cell_index():
    """World::XtoIJK (ch4/World.h:79-92) by the float estimate equals the
    float64 division for random positions and for positions within a few
    ulps of every cell face, on grids near and far from the origin."""
    rng = np.random.default_rng(41)
    for x0, xm, n in [(-0.2, 0.2, 41), (-0.1, 0.1, 21), (0.0, 0.4, 41), (0.0, 0.05, 6), (0.0, 0.4, 512),
                      (1000.0, 1000.5, 101), (-3e-3, 5e-3, 2049)]:
        dh = (xm - x0) / (n - 1)
        ax = dsmc_axis(x0, xm, dh, n - 1)
        x = x0 + rng.random(400_000) * (xm - x0)
        f = x0 + rng.integers(0, n, 40_000) * dh
        near = np.concatenate([f, np.nextafter(f, np.inf), np.nextafter(f, -np.inf), f + dh * 1e-9,
                               f - dh * 1e-9, f + dh * 1e-6, f - dh * 3e-6])
        near = near[(near >= x0) & (near < xm)]
        for xs in (x, near):
            got, want, _ = dsmc_coord(xs, x0, dh, ax)
            assert np.array_equal(got, want), (x0, xm, n)
        if ax[2] < 1:
            assert dsmc_coord(x, x0, dh, ax)[2].mean() > 0.99


def warp_bitonic(vals, R):
    """numpy emulation of warp_bitonic<R> in csrc/k_fp64.cu: element
    i*32 + lane held in a[i] of that lane; exchanges between lanes by
    shuffles (j < 32), within a lane by swaps (j >= 32); INT_MAX pads"""
    a = np.full((R, 32), 2**31 - 1, dtype=np.int64)
    for e, v in enumerate(vals):
        a[e // 32, e % 32] = v
    lanes = np.arange(32)
    k = 2
    while k <= 32 * R:
        j = k >> 1
        while j > 0:
            if j >= 32:
                jj = j >> 5
                for i in range(R):
                    if i & jj == 0:
                        up = ((i * 32 + lanes) & k) == 0
                        x, y = a[i].copy(), a[i | jj].copy()
                        sw = np.where(up, x > y, x < y)
                        a[i], a[i | jj] = np.where(sw, y, x), np.where(sw, x, y)
            else:
                for i in range(R):
                    y = a[i][lanes ^ j]
                    lower = (lanes & j) == 0
                    up = ((i * 32 + lanes) & k) == 0
                    a[i] = np.where(lower == up, np.minimum(a[i], y), np.maximum(a[i], y))
            j >>= 1
        k <<= 1
    return [int(a[e // 32, e % 32]) for e in range(len(vals))]


def test_warp_bitonic_sorts_every_size():
    """the DSMC cell order (k_dsmc_order): each register count R = 1..32
    sorts lists of 2..32R distinct particle indices ascending"""
    rng = np.random.default_rng(1024)
    for R in (1, 2, 4, 8, 16, 32):
        sizes = {2, 16 * R + 1 if R > 1 else 3, 32 * R, int(rng.integers(2, 32 * R + 1))}
        for n in sizes:
            v = rng.choice(1 << 24, n, replace=False)
            assert warp_bitonic(list(v), R) == sorted(v), (R, n)
