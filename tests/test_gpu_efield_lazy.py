"""computeEF of a world whose species are all in the mixed form
(k_efield4): the float copy of E that the mixed push reads, the float64 field
completed on demand, and World::getPE from the same pass.

* The potential is built so that many E components land within a few ulps of
  a float rounding midpoint (the exact-division branch) and the rest do not:
  ions at rest on nodes, pushed once, gain v = q/m E dt from E at their node
  alone, and their float velocities equal those of the same push in a world
  that also holds a float64 species (where k_efield writes both fields).
* The float64 field read back equals the oracle's computeEF of that
  potential bit for bit, also after the potential was overwritten (the
  reference's ef stays that of the last computeEF).
* getPE agrees with the oracle within 1e-13, also on thin grids where most
  of the kernel's threads take face columns.
"""
import numpy as np
import pytest

AMU, QE = 1.660538921e-27, 1.602176565e-19
N = (33, 29, 37)
X0, XM = (-0.1, -0.1, 0.0), (0.1, 0.1, 0.2)


def crafted_phi():
    """phi = A i + B j + C k + noise on a third of the nodes: the differences
    along each axis divided by 2 dh sit at float midpoints (1.5 + 2^-24 and
    friends) to a few float64 ulps where the noise is absent"""
    dh = (np.array(XM) - np.array(X0)) / (np.array(N) - 1)
    mids = [1.5 + 2.0 ** -24, -(3.25 + 2.0 ** -22), 1000.0 * (1 + 2.0 ** -24)]
    A, B, C = (m * d for m, d in zip(mids, dh))
    k, j, i = np.meshgrid(np.arange(N[2]), np.arange(N[1]), np.arange(N[0]), indexing="ij")
    phi = -(A * i + B * j + C * k)
    rng = np.random.default_rng(17)
    noisy = rng.random(phi.shape) < 0.33
    phi = phi + noisy * rng.standard_normal(phi.shape)
    return phi.ravel()


def node_ions(espic, w, n_ions):
    """n_ions at rest on distinct interior nodes, offsets 0 (the push reads E
    at the node alone)"""
    rng = np.random.default_rng(3)
    ii = rng.integers(1, N[0] - 2, n_ions)
    jj = rng.integers(1, N[1] - 2, n_ions)
    kk = rng.integers(1, N[2] - 2, n_ions)
    cell = (ii | (jj << 10) | (kk << 20)).astype(np.int32)
    return cell, np.zeros((3, n_ions), np.float32), np.zeros((3, n_ions), np.float32)


def run(espic, with_fp64):
    with espic.World(*N, X0, XM) as w:
        w.setTime(1e-7, 10)
        s = espic.Species(w, "O+", 16 * AMU, QE, mpw0=1e3, capacity=8192, form=espic.FORM_MIXED)
        if with_fp64:
            espic.Species(w, "e", 9.1e-31, -QE, capacity=64)
        phi = crafted_phi()
        w.write(espic.FIELD_PHI, phi)
        espic.check(espic.lib().espic_efield(w.h))
        cell, off, vel = node_ions(espic, w, 4000)
        s.set_mixed(cell, off, vel)
        s.advance()
        _, _, v = s.get_mixed()
        pe = w.getPE()
        # a new potential (as a solve leaves it) before the first read: the
        # field read is still that of the last computeEF
        w.write(espic.FIELD_PHI, phi + 1.0 + np.arange(phi.size) * 1e-3)
        ef = w.read(espic.FIELD_EF).copy()
        return v, pe, ef, phi


@pytest.mark.gpu
def test_lazy_efield_matches_the_full_one(espic, po):
    v_lazy, pe_lazy, ef_lazy, phi = run(espic, with_fp64=False)
    v_full, pe_full, ef_full, _ = run(espic, with_fp64=True)
    assert np.array_equal(v_lazy.view(np.uint32), v_full.view(np.uint32))
    assert np.count_nonzero(v_lazy) > 3 * 3900
    g = po.grid(list(N), list(X0), list(XM))
    ef_o = po.efield(g, phi).reshape(-1, 3)
    assert np.array_equal(ef_lazy.reshape(-1, 3), ef_o)
    assert np.array_equal(ef_full.reshape(-1, 3), ef_o)
    pe_o = po.potential_energy(g, ef_o, po.node_volumes(g))
    assert abs(pe_lazy - pe_o) <= 1e-13 * abs(pe_o)
    assert abs(pe_full - pe_o) <= 1e-13 * abs(pe_o)


def test_near_midpoint_quotients_occur(po):
    """the crafted potential does exercise the exact-division branch: E
    components whose float64 value lies within 4 ulps of a float midpoint"""
    g = po.grid(list(N), list(X0), list(XM))
    ef = po.efield(g, crafted_phi())
    bits = ef.view(np.uint64) & np.uint64((1 << 29) - 1)
    near = np.abs(bits.astype(np.int64) - (1 << 28)) <= 4
    assert near.sum() > 1000


def run_solved(espic, with_fp64):
    """a sphere world, ions loaded and a float-inner Newton-PCG solve, then
    computeEF (k_efield4 in a mixed-form world, k_efield with the float64
    species)"""
    n = (41, 37, 61)
    x0, xm = (-0.1, -0.1, 0.0), (0.1, 0.1, 0.4)
    with espic.World(*n, x0, xm) as w:
        w.set_seed(5)
        w.setTime(1e-7, 10)
        w.addSphere((0.0, 0.0, 0.15), 0.05, -100.0)
        w.addInlet()
        ions = espic.Species(w, "O+", 16 * AMU, QE, mpw0=2e3, capacity=1 << 19, form=espic.FORM_MIXED,
                             walls=espic.WALLS_ABSORB)
        probe = espic.Species(w, "P+", 16 * AMU, QE, mpw0=1.0, capacity=8192, form=espic.FORM_MIXED)
        if with_fp64:
            espic.Species(w, "e", 9.1e-31, -QE, capacity=64)
        ions.loadParticlesBoxThermal(x0, xm, 0.0, 300000, (0.0, 0.0, 7000.0), 1160.0)
        sol = espic.PotentialSolver(w, espic.SOLVER_PCG, 1000, 1e-4)
        sol.setReferenceValues(0.0, 3.0, 1e10)
        sol.setNewton(nr_max=20, nr_tol=1e-6, pcg_max=2000, pcg_tol=1e-4, fp32_inner=True)
        ions.computeNumberDensity()
        w.computeChargeDensity()
        conv = sol.solve()[0]
        sol.computeEF()
        rng = np.random.default_rng(11)
        m = 4000
        ii, jj, kk = rng.integers(2, n[0] - 3, m), rng.integers(2, n[1] - 3, m), rng.integers(2, n[2] - 3, m)
        probe.set_mixed((ii | (jj << 10) | (kk << 20)).astype(np.int32), np.zeros((3, m), np.float32),
                        np.zeros((3, m), np.float32))
        probe.advance()
        v = probe.get_mixed()[2]
        pe = w.getPE()
        phi = w.phi.copy()
        ef = w.read(espic.FIELD_EF).copy()
        return conv, v, pe, ef, phi, n, x0, xm


@pytest.mark.gpu
def test_efield_after_a_solve_matches_float64(espic, po):
    """after a float-inner solve: the mixed world's float copy equals the
    rounded float64 field of a world where k_efield writes both, the float64
    field equals the oracle's computeEF of the solved phi, and getPE agrees
    within 1e-13"""
    c1, v_pairs, pe_pairs, ef_pairs, phi1, n, x0, xm = run_solved(espic, with_fp64=False)
    c2, v_full, pe_full, ef_full, phi2, _, _, _ = run_solved(espic, with_fp64=True)
    assert c1 and c2
    assert np.array_equal(phi1, phi2)  # the empty float64 species changes nothing in the solve
    assert np.array_equal(v_pairs.view(np.uint32), v_full.view(np.uint32))
    assert np.count_nonzero(v_pairs) > 3 * 3500
    g = po.grid(list(n), list(x0), list(xm))
    ef_o = po.efield(g, phi1).reshape(-1, 3)
    assert np.array_equal(ef_pairs.reshape(-1, 3), ef_o)
    pe_o = po.potential_energy(g, ef_o, po.node_volumes(g))
    assert abs(pe_pairs - pe_o) <= 1e-13 * abs(pe_o)
    assert abs(pe_full - pe_o) <= 1e-13 * abs(pe_o)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [(3, 3, 6), (4, 5, 9), (5, 3, 11), (70, 3, 10)])
def test_thin_grids(espic, po, n):
    """k_efield4 on grids with few interior columns (its threads take the
    interior columns first and the face columns after them): getPE equals
    the oracle's within 1e-13 and the float64 field read back is the
    oracle's computeEF bit for bit"""
    rng = np.random.default_rng(sum(n))
    with espic.World(*n, X0, XM) as w:
        espic.Species(w, "O+", 16 * AMU, QE, mpw0=1e3, capacity=64, form=espic.FORM_MIXED)
        phi = rng.standard_normal(int(np.prod(n)))
        w.write(espic.FIELD_PHI, phi)
        espic.check(espic.lib().espic_efield(w.h))
        pe = w.getPE()
        ef = w.read(espic.FIELD_EF).copy()
    g = po.grid(list(n), list(X0), list(XM))
    ef_o = po.efield(g, phi).reshape(-1, 3)
    assert np.array_equal(ef.reshape(-1, 3), ef_o)
    pe_o = po.potential_energy(g, ef_o, po.node_volumes(g))
    assert abs(pe - pe_o) <= 1e-13 * abs(pe_o)
