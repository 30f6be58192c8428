"""Gradients of the differentiable sphere run (espic_diff_*): no reference
counterpart, so they are pinned by central finite differences of the
forward model and by the float64 adjoint.

The forward model is the sphere step with C1 absorption (a smooth layer of
half a cell inside the sphere and the faces); the loss is the normalised
final field energy plus the normalised ion count of the wake box z in
[0.2, 0.3] m.  Central differences are exact to O(h^2) where the loss is
smooth, but the CIC weights are piecewise linear in position: a step that
moves particles across cell faces averages the slopes on both sides of the
kink.  The sphere potential moves trajectories little, so it is checked at
the relative step 1e-3; drift velocity and initial positions / velocities
(as directional derivatives along a random direction) at 1e-4, where the
kink contribution is below the tolerance.  Tolerance: 1e-4 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE, AMU = 1.602176565e-19, 1.660538921e-27
NODES = (17, 17, 33)
X0, XM = (-0.1, -0.1, 0.0), (0.1, 0.1, 0.3)
N, STEPS, VD, PHI_S = 20000, 40, 7000.0, -100.0


def world(espic, fp32=False):
    w = espic.World(*NODES, X0, XM)
    w.setTime(1e-7, 10 ** 6)
    w.addSphere((0.0, 0.0, 0.15), 0.05, PHI_S)
    w.addInlet()
    sol = espic.PotentialSolver(w, espic.SOLVER_PCG, 100, 1e-4)
    sol.setReferenceValues(0.0, 3.0, 1e10)
    sol.setNewton(nr_max=60, nr_tol=1e-12, pcg_max=5000, pcg_tol=1e-10, fp32_inner=fp32)
    return w


def state(seed=1):
    rng = np.random.default_rng(seed)
    x = np.stack([rng.uniform(-0.09, 0.09, 3 * N), rng.uniform(-0.09, 0.09, 3 * N),
                  rng.uniform(0.01, 0.29, 3 * N)])
    r = np.sqrt(x[0] ** 2 + x[1] ** 2 + (x[2] - 0.15) ** 2)
    x = np.ascontiguousarray(x[:, r > 0.06][:, :N])
    vth = rng.normal(0, 775.0, (3, N))
    return x, vth


def with_drift(vth, vd):
    v = vth.copy()
    v[2] += vd
    return v


def run_args(K=8):
    dh = min(0.2 / 16, 0.3 / 32)
    return dict(n=N, mass=16 * AMU, charge=QE, mpw0=1e10 * 0.012 / N, delta=0.5 * dh, wake_z=(0.2, 0.3),
                checkpoint_every=K)


@pytest.fixture(scope="module")
def setup(espic):
    x0, vth = state()
    w = world(espic)
    with espic.DiffRun(w, alpha=1.0, beta=0.0, **run_args()) as r:
        r.set_state(x0, with_drift(vth, VD))
        pe = r.forward(PHI_S, STEPS)
    with espic.DiffRun(w, alpha=0.0, beta=1.0, **run_args()) as r:
        r.set_state(x0, with_drift(vth, VD))
        m = r.forward(PHI_S, STEPS)
    w.close()
    assert pe > 0 and m > 0
    return x0, vth, 1.0 / pe, 1.0 / m


def gradients(espic, setup, precision="fp64", K=8):
    x0, vth, alpha, beta = setup
    w = world(espic, precision == "fp32")
    with espic.DiffRun(w, alpha=alpha, beta=beta, precision=precision, **run_args(K)) as r:
        r.set_state(x0, with_drift(vth, VD))
        L = r.forward(PHI_S, STEPS)
        g = r.backward()
    w.close()
    return L, g


def rel(a, b):
    return abs(a - b) / abs(b)


def test_gradients_against_central_differences(espic, setup):
    x0, vth, alpha, beta = setup
    L, (dps, dx, dv) = gradients(espic, setup)
    assert abs(L - 2.0) < 1e-12  # both terms normalised to 1
    rng = np.random.default_rng(7)
    dirx, dirv = rng.normal(size=x0.shape), rng.normal(size=x0.shape)
    w = world(espic)
    with espic.DiffRun(w, alpha=alpha, beta=beta, **run_args()) as r:
        def loss(ps=PHI_S, x=x0, v=None):
            r.set_state(x, with_drift(vth, VD) if v is None else v)
            return r.forward(ps, STEPS)

        h = 1e-3
        fd = (loss(ps=PHI_S * (1 + h)) - loss(ps=PHI_S * (1 - h))) / (2 * PHI_S * h)
        assert rel(fd, dps) <= 1e-4, (fd, dps)
        h = 1e-4
        fd = (loss(v=with_drift(vth, VD * (1 + h))) - loss(v=with_drift(vth, VD * (1 - h)))) / (2 * VD * h)
        assert rel(fd, dv[2].sum()) <= 1e-4, (fd, dv[2].sum())
        e = 0.1 * h
        fd = (loss(x=x0 + e * dirx) - loss(x=x0 - e * dirx)) / (2 * e)
        assert rel(fd, (dx * dirx).sum()) <= 1e-4, (fd, (dx * dirx).sum())
        e = 775.0 * h
        v = with_drift(vth, VD)
        fd = (loss(v=v + e * dirv) - loss(v=v - e * dirv)) / (2 * e)
        assert rel(fd, (dv * dirv).sum()) <= 1e-4, (fd, (dv * dirv).sum())
    w.close()


def test_fp32_adjoint_against_fp64(espic, setup):
    L64, (p64, x64, v64) = gradients(espic, setup, "fp64")
    L32, (p32, x32, v32) = gradients(espic, setup, "fp32")
    assert rel(L32, L64) <= 1e-6
    assert rel(p32, p64) <= 1e-4
    assert rel(v32[2].sum(), v64[2].sum()) <= 1e-4
    rng = np.random.default_rng(3)
    d = rng.normal(size=x64.shape)
    assert rel((x32 * d).sum(), (x64 * d).sum()) <= 1e-4
    assert rel((v32 * d).sum(), (v64 * d).sum()) <= 1e-4


def test_checkpoint_interval_does_not_change_gradients(espic, setup):
    _, (p8, x8, v8) = gradients(espic, setup, K=8)
    _, (p40, x40, v40) = gradients(espic, setup, K=40)
    assert rel(p40, p8) <= 1e-10
    assert np.max(np.abs(x40 - x8)) <= 1e-9 * np.max(np.abs(x8))
    assert np.max(np.abs(v40 - v8)) <= 1e-9 * np.max(np.abs(v8))


def test_torch_autograd_function(espic, setup):
    torch = pytest.importorskip("torch")
    x0, vth, alpha, beta = setup
    _, (dps, dx, dv) = gradients(espic, setup)
    w = world(espic)
    with espic.DiffRun(w, alpha=alpha, beta=beta, **run_args()) as r:
        ps = torch.tensor(PHI_S, dtype=torch.float64, requires_grad=True)
        vd = torch.tensor(VD, dtype=torch.float64, requires_grad=True)
        x = torch.tensor(x0, dtype=torch.float64, requires_grad=True)
        zhat = torch.tensor([0.0, 0.0, 1.0], dtype=torch.float64)[:, None]
        v = torch.tensor(vth, dtype=torch.float64) + vd * zhat
        loss = espic.sphere_run_loss(r, ps, x, v, STEPS)
        loss.backward()
    w.close()
    assert rel(ps.grad.item(), dps) <= 1e-12
    assert rel(vd.grad.item(), dv[2].sum()) <= 1e-12
    assert np.allclose(x.grad.numpy(), dx, rtol=0, atol=1e-12 * np.max(np.abs(dx)))


def test_full_scale_gradients_converge(espic):
    """The 32x32x64 box, 500k ions, 400 steps, checkpoints every 20: over this
    horizon the loss is linear only at small relative scales (perturbations
    grow through the dynamics), so the central difference uses h = 1e-7."""
    n, steps = 500_000, 400
    rng = np.random.default_rng(11)
    lo, hi, c = np.array(X0), np.array(XM), np.array([0.0, 0.0, 0.15])
    pos = lo + rng.random((3 * n, 3)) * (hi - lo)
    pos = pos[np.sum((pos - c) ** 2, axis=1) > 0.055 ** 2][:n]
    x = np.ascontiguousarray(pos.T)
    vth = rng.normal(0, 775.0, (3, n))
    geo = (32, 32, 64)
    dh = min(0.2 / 31, 0.3 / 63)

    def mk():
        w = espic.World(*geo, X0, XM)
        w.setTime(1e-7, 10 ** 6)
        w.addSphere((0.0, 0.0, 0.15), 0.05, PHI_S)
        w.addInlet()
        sol = espic.PotentialSolver(w, espic.SOLVER_PCG, 100, 1e-4)
        sol.setReferenceValues(0.0, 3.0, 1e10)
        sol.setNewton(nr_max=60, nr_tol=1e-12, pcg_max=5000, pcg_tol=1e-10, fp32_inner=False)
        return w

    kw = dict(n=n, mass=16 * AMU, charge=QE, mpw0=1e10 * 0.0115 / n, delta=0.5 * dh, wake_z=(0.2, 0.3),
              checkpoint_every=20)
    w = mk()
    with espic.DiffRun(w, alpha=1e8, beta=1e-7, **kw) as r:
        def loss(ps=PHI_S, v=None):
            r.set_state(x, with_drift(vth, VD) if v is None else v)
            return r.forward(ps, steps)

        loss()
        dps, _, dv = r.backward()
        h = 1e-7
        fd = (loss(ps=PHI_S * (1 + h)) - loss(ps=PHI_S * (1 - h))) / (2 * PHI_S * h)
        assert rel(fd, dps) <= 1e-4, (fd, dps)
        fd = (loss(v=with_drift(vth, VD * (1 + h))) - loss(v=with_drift(vth, VD * (1 - h)))) / (2 * VD * h)
        assert rel(fd, dv[2].sum()) <= 1e-4, (fd, dv[2].sum())
    w.close()
