"""Failure detection through status codes, with faults made on the host (no
GPU fault, trap or hang): a particle whose position is NaN and a charge
density holding a NaN.  The kernels flag the non-finite value on the device;
the next call that synchronises returns ESPIC_ERR_NONFINITE with its
message, clears the flag, and the world stays usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

AMU, QE = 1.660538921e-27, 1.602176565e-19
ERR_NONFINITE = -4
BOX = ([21, 21, 21], [-0.1, -0.1, 0.0], [0.1, 0.1, 0.2])


def test_nan_particle_is_reported_and_removed(espic):
    rng = np.random.default_rng(4)
    with espic.World(*BOX[0], BOX[1], BOX[2]) as w:
        w.setTime(2e-10, 10)
        s = espic.Species(w, "O+", 16 * AMU, QE, mpw0=1.0, capacity=64, form=espic.FORM_FP64,
                          walls=espic.WALLS_ABSORB)
        P = np.zeros((7, 10))
        P[0:2] = -0.05 + 0.1 * rng.random((2, 10))
        P[2] = 0.05 + 0.1 * rng.random(10)
        P[6] = 1.0
        P[0, 3] = np.nan
        s.set_particles(P)
        s.advance()
        with pytest.raises(espic.EspicError) as e:
            s.getNp()
        assert e.value.code == ERR_NONFINITE
        # the flag is cleared; the NaN particle was removed, the others kept
        assert s.getNp() == 9
        got = s.particles()
        keep = np.isfinite(P[0])
        assert np.array_equal(np.sort(got[0]), np.sort(P[0, keep]))


def test_nan_charge_density_stops_the_solve(espic):
    with espic.World(*BOX[0], BOX[1], BOX[2]) as w:
        rho = np.full(w.nn, 1e-9)
        rho[w.nn // 2] = np.nan
        w.write(espic.FIELD_RHO, rho)
        solver = espic.PotentialSolver(w, espic.SOLVER_SOR, 10000, 1e-4)
        with pytest.raises(espic.EspicError) as e:
            solver.solve()
        assert e.value.code == ERR_NONFINITE
        # a finite density solves afterwards on the same world
        w.write(espic.FIELD_PHI, np.zeros(w.nn))
        w.write(espic.FIELD_RHO, np.full(w.nn, 1e-9))
        conv = solver.solve()[0]
        assert conv
