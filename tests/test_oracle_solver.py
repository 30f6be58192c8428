"""The oracle's Newton-PCG with the reference's fallback: when the inner
linear PCG fails (here: capped at 2 iterations) the reference continues with
Gauss-Seidel on the same linear system (ch3/ver2/PotentialSolver.cpp:270-271,
solveGSLinear :433-461).  CPU only."""
import numpy as np

SPH = ([17, 17, 33], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.4])


def problem(po):
    g = po.grid(*SPH)
    obj, phi = po.objects(g, [0.0, 0.0, 0.15], 0.05, -100.0)
    rho = 1e10 * 1.602176565e-19 * (1 + 0.1 * np.random.default_rng(1).random(g.nn))
    return g, obj, phi, rho


def test_fallback_converges_to_the_tight_solution(po):
    g, obj, phi, rho = problem(po)
    tight, conv, _, _ = po.newton_pcg(g, phi, rho, obj, 0.0, 3.0, 1e10, 50, 1e-11, 20000, 1e-12)
    assert conv
    got, conv, nr, pcg, gs = po.newton_pcg_fallback(g, phi, rho, obj, 0.0, 3.0, 1e10, 50, 1e-8, 2, 1e-12, 20000, 1e-6)
    assert conv and gs > 0 and pcg <= 2 * nr
    assert np.max(np.abs(got - tight)) <= 1e-8 * np.max(np.abs(tight))


def test_without_fallback_the_capped_solve_fails(po):
    g, obj, phi, rho = problem(po)
    _, conv, nr, pcg, gs = po.newton_pcg_fallback(g, phi, rho, obj, 0.0, 3.0, 1e10, 5, 1e-8, 2, 1e-12, 0, 1e-6)
    assert not conv and gs == 0 and nr == 5
