// Output written against the reference's API: the sphere run of
// sphere_main.cpp calling Output::fields every 5 steps (ch3/ver2/Main.cpp:
// 81-83), Output::diagOutput every step and Output::screenOutput.
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "World.h"
#include "Species.h"
#include "PotentialSolver.h"
#include "Source.h"
#include "Output.h"

int main(int argc, char **argv) {
    int steps = argc > 1 ? atoi(argv[1]) : 10;
    World world(21, 21, 41);
    world.setExtents({-0.1, -0.1, 0}, {0.1, 0.1, 0.4});
    world.setTime(1e-7, steps);
    world.addSphere({0, 0, 0.15}, 0.05, -100);
    world.addInlet();
    std::vector<Species> species;
    species.push_back(Species("O+", 16 * Const::AMU, Const::QE, 5e2, world));
    std::vector<ColdBeamSource> sources;
    sources.push_back(ColdBeamSource(species[0], world, 7000, 1e10));
    PotentialSolver solver(world, SolverType::GS, 20000, 1e-4);
    solver.setReferenceValues(0, 1.5, 1e10);
    solver.solve();
    solver.computeEF();
    while (world.advanceTime()) {
        for (ColdBeamSource &s : sources) s.sample();
        for (Species &sp : species) {
            sp.advance();
            sp.computeNumberDensity();
            sp.updateAverages();
        }
        world.computeChargeDensity(species);
        solver.solve();
        solver.computeEF();
        if (world.getTs() % 5 == 0 || world.isLastTimeStep()) {
            Output::screenOutput(world, species);
            Output::fields(world, species);
        }
    }
    return 0;
}
