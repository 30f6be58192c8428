/*
 * PotentialSolver.h (drop-in) -- the reference's PotentialSolver
 * (ch2/PotentialSolver.h:6-23 and ch3/ver2/PotentialSolver.h:42-104, with
 * the GSCUDA type of ch9/CUDA/PotentialSolver.h:8) on libespic.
 *
 * The ch2 constructor (world, max_it, tol) selects the linear red-black SOR
 * with Dirichlet walls.  The ch3 constructor (world, type, max_it, tol)
 * selects the Boltzmann-electron solvers: GS (and GSCUDA) -> red-black
 * nonlinear SOR, PCG -> Newton with the multigrid-preconditioned CG,
 * QN -> quasi-neutral inversion.  As in the reference, constructing a ch3
 * solver runs the quasi-neutral solve once (buildMatrix ends in solveQN).
 */
#ifndef ESPIC_SHIM_POTENTIALSOLVER_H
#define ESPIC_SHIM_POTENTIALSOLVER_H

#include "World.h"

enum SolverType { GS, PCG, QN, GSCUDA };

class PotentialSolver {
public:
    PotentialSolver(World &world, int max_it, double tol);
    PotentialSolver(World &world, SolverType type, int max_it, double tol);

    void setReferenceValues(double phi0, double Te0, double n0) {
        this->phi0 = phi0;
        this->Te0 = Te0;
        this->n0 = n0;
    }
    bool solve();
    void computeEF();
    void buildMatrix();
    /* ch9/CUDA: phi stays on the GPU; the host mirror pulls it on access */
    void updateHostPhi() { world.phi.pull(); }

protected:
    World &world;
    int kind;
    unsigned max_solver_it;
    double tolerance;
    double phi0 = 0;
    double n0 = 1e12;
    double Te0 = 1.5;
    void configure();
};

#endif
