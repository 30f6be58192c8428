/* ch4_api_main.cpp -- uses the ch4 World / vec3 / Species / Collisions API of
 * the drop-in headers (compiled by tests/test_drop_in.py; run on a GPU it
 * prints the host geometry helpers and one DSMC and MCC call). */
#include <iostream>
#include <memory>
#include <vector>

#include "Collisions.h"
#include "Output.h"
#include "PotentialSolver.h"
#include "Source.h"
#include "Species.h"
#include "World.h"

using namespace Const;

int main() {
    World world(21, 11, 21);
    world.setExtents({-0.2, -0.1, 0}, {0.2, 0.1, 0.4});
    world.setTime(1e-7, 10);
    world.addSphere({0, 0, 0.15}, 0.05, -100);
    double3 a{0, 0, 0.0}, b{0, 0, 0.3};
    std::cout << world.XtoC({0.01, 0.01, 0.01}) << " " << world.XtoIJK({0.01, 0.01, 0.01})[2] << " "
              << world.lineSphereIntersect(a, b) << " " << mag(world.sphereDiffuseVector({0, 0, 0.1})) << " "
              << dot(cross(a, b), unit(b)) << std::endl;
    std::vector<Species> species;
    species.push_back(Species("O", 16 * AMU, 0, 1e12, world));
    species.push_back(Species("O+", 16 * AMU, QE, 5e1, world));
    Species &neutrals = species[0];
    Species &ions = species[1];
    std::vector<std::unique_ptr<Interaction>> interactions;
    interactions.emplace_back(new DSMC_MEX(neutrals, world));
    interactions.emplace_back(new MCC_CEX(ions, neutrals, world));
    WarmBeamSource source(neutrals, world, 7000, 2e20, 1000);
    while (world.advanceTime()) {
        source.sample();
        neutrals.computeNumberDensity();
        neutrals.sampleMoments();
        neutrals.computeGasProperties();
        for (auto &i : interactions) i->apply(world.getDt());
        neutrals.advance(neutrals, neutrals);
        neutrals.computeMPC();
    }
    std::cout << neutrals.getNp() << " " << neutrals.T(10, 5, 10) << " " << neutrals.mpc(1, 1, 1) << std::endl;
    return 0;
}
