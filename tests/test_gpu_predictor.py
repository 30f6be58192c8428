"""The Newton solve's predictor (espic_solver_set_predictor): between
consecutive solves the float-inner solve starts from an extrapolation in
time of the last potentials, 2 phi^n - phi^(n-1) after two solves and
3 phi^n - 3 phi^(n-1) + phi^(n-2) from the third on.

* A charge density that varies smoothly from one solve to the next: the
  potentials with and without the predictor agree to far inside the Newton
  tolerance (the converged solution does not depend on the start), and the
  predicted solves need fewer inner iterations.
* Two density writes between solves (not consecutive) and a potential
  written by hand both restart the history: the solves still agree.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

QE = 1.602176565e-19
N = (41, 37, 61)
X0, XM = (-0.1, -0.1, 0.0), (0.1, 0.1, 0.4)


def density(n):
    """rho at solve n: the ion density 1e10 m^-3 modulated smoothly in space
    and in time"""
    k, j, i = np.meshgrid(np.arange(N[2]), np.arange(N[1]), np.arange(N[0]), indexing="ij")
    z = k / (N[2] - 1)
    x = i / (N[0] - 1)
    return (QE * 1e10 * (1.0 + 0.3 * np.sin(0.25 * n + 6.0 * z)) * (1.0 + 0.1 * x)).ravel()


def world(espic, predictor):
    w = espic.World(*N, X0, XM)
    w.setTime(1e-7, 100)
    w.addSphere((0.0, 0.0, 0.15), 0.05, -100.0)
    w.addInlet()
    espic.Species(w, "O+", 16 * 1.660538921e-27, QE, mpw0=1e3, capacity=1024, form=espic.FORM_MIXED)
    sol = espic.PotentialSolver(w, espic.SOLVER_PCG, 1000, 1e-4)
    sol.setReferenceValues(0.0, 3.0, 1e10)
    sol.setNewton(nr_max=20, nr_tol=1e-6, pcg_max=2000, pcg_tol=1e-4, fp32_inner=True)
    sol.setPredictor(predictor)
    return w, sol


def run(espic, predictor, schedule):
    """schedule: per solve, the densities written before it (several writes:
    not consecutive) and whether phi is overwritten first"""
    w, sol = world(espic, predictor)
    phis, inner = [], []
    with w:
        for writes, touch_phi in schedule:
            if touch_phi:
                w.write(espic.FIELD_PHI, w.phi.copy())
            for n in writes:
                w.write(espic.FIELD_RHO, density(n))
            conv, _, it, _ = sol.solve()
            assert conv
            phis.append(w.phi.copy())
            inner.append(it)
    return phis, inner


def test_predicted_solves_match_and_save_iterations(espic):
    schedule = [([n], False) for n in range(8)]
    p_on, it_on = run(espic, True, schedule)
    p_off, it_off = run(espic, False, schedule)
    for a, b in zip(p_on, p_off):
        assert np.max(np.abs(a - b)) < 1e-5
    # the first solve has no history; from the third the quadratic formula
    assert it_on[0] == it_off[0]
    assert sum(it_on[3:]) < sum(it_off[3:])


def test_history_restarts(espic):
    schedule = [([0], False), ([1], False), ([2], False), ([3, 4], False), ([5], False), ([6], True),
                ([7], False), ([8], False)]
    p_on, _ = run(espic, True, schedule)
    p_off, _ = run(espic, False, schedule)
    for a, b in zip(p_on, p_off):
        assert np.max(np.abs(a - b)) < 1e-5
