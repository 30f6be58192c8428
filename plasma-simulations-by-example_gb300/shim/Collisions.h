/*
 * Collisions.h (drop-in) -- the material interactions of the reference
 * (ch4/Collisions.h:33-89) on libespic: DSMC_MEX (neutral-neutral
 * collisions), MCC_CEX (charge exchange) and ChemistryIonize (ions created
 * from the neutral density and rho) run on the GPU.
 */
#ifndef ESPIC_SHIM_COLLISIONS_H
#define ESPIC_SHIM_COLLISIONS_H

#include "Species.h"
#include "World.h"

class Interaction {
public:
    virtual void apply(double dt) = 0;
    virtual ~Interaction() {}
};

/* MCC_CEX::apply, ch4/Collisions.cpp:43-80 */
class MCC_CEX : public Interaction {
public:
    MCC_CEX(Species &source, Species &target, World &world) : source{source}, target{target}, world{world} {}
    void apply(double dt);

protected:
    Species &source;
    Species &target;
    World &world;
};

/* DSMC_MEX::apply, ch4/Collisions.cpp:108-183 (VHS parameters of the
 * reference's constructor, sigma_cr_max starting at 1e-14) */
class DSMC_MEX : public Interaction {
public:
    DSMC_MEX(Species &species, World &world);
    void apply(double dt);
    double sigmaCrMax();

protected:
    Species &species;
    World &world;
};

/* ChemistryIonize::apply, ch4/Collisions.cpp:10-31 */
class ChemistryIonize : public Interaction {
public:
    ChemistryIonize(Species &neutrals, Species &ions, World &world, double rate)
        : neutrals{neutrals}, ions{ions}, world{world}, rate{rate} {}
    void apply(double dt);

protected:
    Species &neutrals;
    Species &ions;
    World &world;
    double rate;
};

#endif
