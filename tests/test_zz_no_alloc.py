"""espic_deposit_noalloc, the deposit entry point for callers that may not
allocate device memory (a host whose pool allocator already owns the GPU's
memory, a real-time loop that forbids allocation after start-up, code that
must not synchronise the device).  Through the C-ABI, with device buffers
the caller owns, two calls in a row must each give exactly the density of
the allocating entry point, espic_deposit (bit-for-bit, the tolerance this
suite uses for fixed-point charge).  The two agree bit for bit because the
allocating species here has a capacity equal to the particle count: both
entry points then pick the same fixed-point scale.

This file is named so that pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

QE, AMU, ME = 1.602176565e-19, 1.660538921e-27, 9.10938215e-31
GRID = (21, 21, 21)
X0, XM = (-0.1, -0.1, 0.0), (0.1, 0.1, 0.2)


def entry(espic):
    f = espic.lib().espic_deposit_noalloc
    f.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double),
                  C.POINTER(C.c_double), C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
    f.restype = C.c_int
    return f


def d3(v):
    return (C.c_double * 3)(*v)


def allocating_deposit(espic, P, mass, charge, weight_bound):
    # capacity == n: the scale espic_deposit_noalloc derives from n
    with espic.World(*GRID, X0, XM) as w:
        s = espic.Species(w, "s", mass, charge, capacity=P.shape[1], weight_bound=weight_bound)
        s.set_particles(P)
        s.computeNumberDensity()
        return s.den


def test_noalloc_matches_allocating_deposit_on_two_calls(espic):
    import torch
    f = golden("box_deposit")
    fn = entry(espic)
    nn = GRID[0] * GRID[1] * GRID[2]
    den = torch.full((nn,), float("nan"), dtype=torch.float64, device="cuda")
    flags = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    # two calls in a row with different particles: the second must not see
    # the first call's sums left in the shared scratch
    for P, mass, q in ((f["Pi"], 16 * AMU, QE), (f["Pe"], ME, -QE)):
        n = P.shape[1]
        wb = float(P[6].max())
        want = allocating_deposit(espic, P, mass, q, wb)
        dP = torch.from_numpy(np.ascontiguousarray(P)).to("cuda")
        torch.cuda.synchronize()
        rc = fn(dP.data_ptr(), n, n, *GRID, d3(X0), d3(XM), wb, den.data_ptr(), flags.data_ptr(),
                stream.cuda_stream)
        assert rc == 0, espic.last_error()
        torch.cuda.synchronize()
        got = den.cpu().numpy()
        assert np.array_equal(got, want)
        assert int(flags.item()) == 0


def test_noalloc_flags_and_skips_particles_it_cannot_sum(espic):
    """A weight above weight_bound (it could wrap the int64 sums) and a NaN
    position deposit nothing and set their bits in the caller's flag word,
    where the allocating path returns ESPIC_ERR_FIXED / ESPIC_ERR_NONFINITE;
    the other particles give the allocating path's density."""
    import torch
    f = golden("box_deposit")
    fn = entry(espic)
    P = np.ascontiguousarray(f["Pi"][:, :2000])
    n = P.shape[1]
    wb = float(P[6].max())
    Q = np.concatenate([P, P[:, :2]], axis=1)
    Q[6, n] = 4 * wb
    Q[0, n + 1] = np.nan
    nn = GRID[0] * GRID[1] * GRID[2]
    den = torch.zeros(nn, dtype=torch.float64, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    dQ = torch.from_numpy(Q).to("cuda")
    torch.cuda.synchronize()
    # the allocating path on the same n + 2 slots (same fixed-point scale),
    # with the two bad particles replaced by zero weights that add nothing
    want = allocating_deposit(espic, np.concatenate([P, P[:, :2] * 0], axis=1), 16 * AMU, QE, wb)
    rc = fn(dQ.data_ptr(), n + 2, n + 2, *GRID, d3(X0), d3(XM), wb, den.data_ptr(), flags.data_ptr(),
            torch.cuda.current_stream().cuda_stream)
    assert rc == 0, espic.last_error()
    torch.cuda.synchronize()
    assert int(flags.item()) == 3  # ESPIC_NOALLOC_RANGE | ESPIC_NOALLOC_NONFINITE
    assert np.array_equal(den.cpu().numpy(), want)


def test_noalloc_refuses_grids_beyond_its_scratch(espic):
    import torch
    fn = entry(espic)
    den = torch.zeros(8, dtype=torch.float64, device="cuda")
    rc = fn(None, 0, 0, 128, 128, 128, d3(X0), d3(XM), 1.0, den.data_ptr(), None, None)
    assert rc == -1
    assert "scratch" in espic.last_error()
