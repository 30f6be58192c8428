/*
 * Species.h (drop-in) -- the Species class of the reference
 * (ch2/Species.h:22-65, ch3/ver2/Species.h:22-72, ch4/Species.h:22-96) on
 * libespic.
 *
 * The particles live on the GPU.  The public `particles` member is a host
 * mirror with the std::vector<Particle> operations the reference's code uses;
 * it is refreshed from the device on first access after device work and its
 * edits are pushed back before the next device operation.
 * advance() followed by computeNumberDensity() runs as one fused push +
 * deposit kernel.
 */
#ifndef ESPIC_SHIM_SPECIES_H
#define ESPIC_SHIM_SPECIES_H

#include <string>
#include <vector>

#include "Field.h"
#include "World.h"

struct Particle {
    double3 pos;
    double3 vel;
    double mpw;
    Particle(double3 x, double3 v, double mpw) : pos{x}, vel{v}, mpw{mpw} {}
};

class Species;

/* host mirror of a species' device particle store */
class ParticleVector {
public:
    typedef std::vector<Particle>::iterator iterator;
    size_t size() { return host().size(); }
    bool empty() { return host().empty(); }
    Particle &operator[](size_t i) { return edit()[i]; }
    Particle &back() { return edit().back(); }
    iterator begin() { return edit().begin(); }
    iterator end() { return edit().end(); }
    void reserve(size_t n) { v.reserve(n); }
    void clear() { edit().clear(); }
    void push_back(const Particle &p) { edit().push_back(p); }
    template <class... A>
    void emplace_back(A &&...a) {
        edit().emplace_back(std::forward<A>(a)...);
    }
    iterator erase(iterator a, iterator b) { return edit().erase(a, b); }

    Species *owner = nullptr;
    bool host_valid = true;  /* mirror equals the device */
    bool host_dirty = false; /* mirror edited since the last push */

private:
    std::vector<Particle> &host();
    std::vector<Particle> &edit() {
        host();
        host_dirty = true;
        return v;
    }
    std::vector<Particle> v;
    friend class Species;
};

class Species {
public:
    /* ch2: weights from the loaders; particles reflect off the walls */
    Species(std::string name, double mass, double charge, World &world);
    /* ch3: default weight mpw0; particles leave through the walls */
    Species(std::string name, double mass, double charge, double mpw0, World &world);
    Species(Species &&o) noexcept;
    Species(const Species &) = delete;

    size_t getNp();
    double getRealCount();
    double3 getMomentum();
    double getKE();
    void advance();
    void computeNumberDensity();
    void addParticle(double3 pos, double3 vel, double mpwt);
    void addParticle(double3 pos, double3 vel) { addParticle(pos, vel, mpw0); }
    /* ch4/Species.h:67: the library keeps no per-particle time; a particle
     * added here has one dt left at the next ch4 push, whatever dt says */
    void addParticle(double3 pos, double3 vel, double dt, double mpw) {
        (void)dt;
        addParticle(pos, vel, mpw);
    }
    void loadParticlesBox(double3 x1, double3 x2, double num_den, int num_mp);
    void loadParticlesBoxQS(double3 x1, double3 x2, double num_den, int3 num_mp);
    void updateAverages();
    /* ch4/Species.cpp:149-175 */
    double sampleVth(double T);
    double3 sampleIsotropicVel(double T);
    /* ch4 (ch4/Species.h:47-62): the push of a neutral species with the
     * sphere's diffuse reflection (charged species: not built), moments,
     * gas properties and macroparticles per cell */
    void advance(Species &neutrals, Species &spherium);
    void sampleMoments();
    void computeGasProperties();
    void computeMPC();
    void clearSamples();

    const std::string name;
    const double mass;
    const double charge;
    const double mpw0;

    ParticleVector particles;
    Field den;
    Field den_ave;
    Field T;    /* ch4: temperature (computeGasProperties) */
    Field3 vel; /* ch4: stream velocity */
    Field mpc;  /* ch4: macroparticles per cell, (ni-1)(nj-1)(nk-1) */

    /* ---- libespic plumbing ---- */
    int id() const { return sid; }
    void settle();               /* run a pending push, push host particle edits */
    void particles_changed();    /* device work moved or changed the particles */
    void pull_particles(std::vector<Particle> &out);
    World &get_world() { return world; }

protected:
    World &world;
    int sid = -1;
    bool push_pending = false;
    void create(int walls);
    void bind_fields();
    double diag[5] = {0, 0, 0, 0, 0};
    bool diag_valid = false;
    void refresh_diag();
};

#endif
