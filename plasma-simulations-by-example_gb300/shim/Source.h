/*
 * Source.h (drop-in) -- ColdBeamSource (ch3/ver2/Source.h:8-21) and
 * WarmBeamSource (ch4/Source.h:32-46) on libespic: particles are generated on
 * the GPU from the world's Philox streams.
 */
#ifndef ESPIC_SHIM_SOURCE_H
#define ESPIC_SHIM_SOURCE_H

#include "Species.h"
#include "World.h"

class Source {
public:
    virtual void sample() = 0;
    virtual ~Source() {}
};

class ColdBeamSource : public Source {
public:
    ColdBeamSource(Species &species, World &world, double v_drift, double den)
        : sp{species}, world{world}, v_drift{v_drift}, den{den} {}
    void sample();

protected:
    Species &sp;
    World &world;
    double v_drift;
    double den;
    int src = -1;
    double temperature() const { return 0; }
};

class WarmBeamSource : public Source {
public:
    WarmBeamSource(Species &species, World &world, double v_drift, double den, double T)
        : sp{species}, world{world}, v_drift{v_drift}, den{den}, T{T} {}
    void sample();

protected:
    Species &sp;
    World &world;
    double v_drift;
    double den;
    double T;
    int src = -1;
};

#endif
