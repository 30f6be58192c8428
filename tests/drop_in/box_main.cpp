// A grounded-box run written against the reference's class API (World,
// Species, PotentialSolver, Output) and built with the drop-in headers:
// two species loaded at random, an initial solve, then N steps of the
// ch2-style loop, printing the diagnostics row of every step.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "World.h"
#include "Species.h"
#include "PotentialSolver.h"

int main(int argc, char **argv) {
    int steps = argc > 1 ? atoi(argv[1]) : 10;
    World world(21, 21, 21);
    world.setExtents({-0.1, -0.1, 0}, {0.1, 0.1, 0.2});
    world.setTime(2e-10, steps);
    std::vector<Species> species;
    species.reserve(2);
    species.push_back(Species("O+", 16 * Const::AMU, Const::QE, world));
    species.push_back(Species("e-", Const::ME, -1 * Const::QE, world));
    species[0].loadParticlesBox(world.getX0(), world.getXm(), 1e11, 20000);
    species[1].loadParticlesBox(world.getX0(), world.getXc(), 1e11, 5000);
    PotentialSolver solver(world, 10000, 1e-4);
    solver.solve();
    solver.computeEF();
    while (world.advanceTime()) {
        for (Species &sp : species) {
            sp.advance();
            sp.computeNumberDensity();
        }
        world.computeChargeDensity(species);
        solver.solve();
        solver.computeEF();
        printf("%d", world.getTs());
        for (Species &sp : species) {
            double3 m = sp.getMomentum();
            printf(" %zu %.17g %.17g %.17g %.17g %.17g", sp.getNp(), sp.getRealCount(), m[0], m[1], m[2], sp.getKE());
        }
        printf(" %.17g\n", world.getPE());
    }
    // host mirrors: phi and one particle, pulled from the device
    printf("phi %.17g\n", world.phi(10, 10, 10));
    Particle &p = species[1].particles[7];
    printf("p %.17g %.17g %.17g\n", p.pos[0], p.vel[1], p.mpw);
    return 0;
}
