/* ch4_ions_main.cpp -- a ch4 plasma written against the reference's class
 * API (compiled by tests/test_drop_in.py): neutral and ion beams, ions
 * striking the sphere (Species::advance(neutrals, spherium) of a charged
 * species) add neutrals and sputtered atoms, sputtered atoms are ionized
 * (ChemistryIonize) and ions charge-exchange with the neutrals (MCC_CEX).
 * Prints per step: ts, then each species' count. */
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <vector>

#include "Collisions.h"
#include "PotentialSolver.h"
#include "Source.h"
#include "Species.h"
#include "World.h"

using namespace Const;

int main(int argc, char **argv) {
    const int steps = argc > 1 ? atoi(argv[1]) : 10;
    World world(21, 11, 21);
    world.setExtents({-0.2, -0.1, 0}, {0.2, 0.1, 0.4});
    world.setTime(1e-6, steps);
    world.addSphere({0, 0, 0.15}, 0.05, -100);
    world.addInlet();

    std::vector<Species> species;
    /* two neutrals and, above 5000 m/s, two sputtered atoms per ion strike */
    species.push_back(Species("O", 16 * AMU, 0, 1e5, world));
    species.push_back(Species("O+", 16 * AMU, QE, 2e5, world));
    species.push_back(Species("Sph", 100 * AMU, 0, 1e4, world));
    species.push_back(Species("Sph+", 100 * AMU, QE, 1e4, world));
    Species &neutrals = species[0];
    Species &ions = species[1];
    Species &sph = species[2];
    Species &sph_ions = species[3];

    std::vector<std::unique_ptr<Source>> sources;
    sources.emplace_back(new WarmBeamSource(neutrals, world, 7000, 1e14, 1000));
    sources.emplace_back(new ColdBeamSource(ions, world, 7000, 1e12));

    std::vector<std::unique_ptr<Interaction>> interactions;
    interactions.emplace_back(new ChemistryIonize(sph, sph_ions, world, 1e-11));
    interactions.emplace_back(new MCC_CEX(ions, neutrals, world));

    PotentialSolver solver(world, SolverType::GS, 2000, 1e-4);
    solver.setReferenceValues(0, 1.5, 1e12);
    solver.solve();
    solver.computeEF();

    while (world.advanceTime()) {
        for (auto &s : sources) s->sample();
        for (auto &i : interactions) i->apply(world.getDt());
        for (Species &sp : species) {
            sp.advance(neutrals, sph);
            sp.computeNumberDensity();
        }
        world.computeChargeDensity(species);
        /* as ch4/Main.cpp: the potential of the initial solve, E each step */
        solver.computeEF();
        printf("%d", world.getTs());
        for (Species &sp : species) printf(" %zu", sp.getNp());
        printf("\n");
    }
    return 0;
}
