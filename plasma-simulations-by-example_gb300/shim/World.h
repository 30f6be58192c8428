/*
 * World.h (drop-in) -- the World class of the reference (ch2/World.h:38-110,
 * ch3/ver2/World.h:38-147, ch9/MT/World.h setNumThreads) on libespic.
 *
 * The device copy of phi, rho, node_vol, ef and object_id is authoritative;
 * the public Field members are lazily synchronised host mirrors.  The GPU
 * world is created by setExtents (the C-ABI needs the extents).
 */
#ifndef ESPIC_SHIM_WORLD_H
#define ESPIC_SHIM_WORLD_H

#include <chrono>
#include <random>
#include <vector>

#include "Field.h"

struct espic_world;
class Species;

namespace Const {
const double EPS_0 = 8.85418782e-12;
const double QE = 1.602176565e-19;
const double AMU = 1.660538921e-27;
const double ME = 9.10938215e-31;
const double K = 1.380648e-23;
const double PI = 3.141592653;
const double EvToK = QE / K;
}  // namespace Const

/* host random numbers with the reference's interface (ch2/World.h:24-33);
 * the GPU samplers draw from Philox streams of the world instead */
class Rnd {
public:
    Rnd() : mt_gen{std::random_device()()}, rnd_dist{0, 1.0} {}
    double operator()() { return rnd_dist(mt_gen); }

protected:
    std::mt19937 mt_gen;
    std::uniform_real_distribution<double> rnd_dist;
};

extern Rnd rnd;

class World {
public:
    World(int ni, int nj, int nk);
    ~World();
    World(const World &) = delete;
    World &operator=(const World &) = delete;

    void setExtents(const double3 x0, const double3 xm);
    double3 getX0() const { return double3(x0); }
    double3 getXm() const { return double3(xm); }
    double3 getXc() const { return double3(xc); }
    double3 getDh() const { return double3(dh); }
    double getCellVolume() const { return dh(0) * dh(1) * dh(2); }

    int getTs() const { return ts; }
    double getTime() const { return time; }
    double getWallTime();
    double getDt() const { return dt; }
    bool isLastTimeStep() const { return ts == num_ts - 1; }

    bool inBounds(double3 pos) {
        for (int i = 0; i < 3; i++)
            if (pos[i] < x0[i] || pos[i] >= xm[i]) return false;
        return true;
    }

    void setTime(double dt, int num_ts);
    bool advanceTime();

    double3 XtoL(double3 x) const {
        double3 lc;
        lc[0] = (x[0] - x0(0)) / dh(0);
        lc[1] = (x[1] - x0(1)) / dh(1);
        lc[2] = (x[2] - x0(2)) / dh(2);
        return lc;
    }
    double3 pos(double3 lc) {
        double3 x = x0 + dh * lc;
        return x;
    }
    double3 pos(int i, int j, int k) {
        double3 x{(double)i, (double)j, (double)k};
        return pos(x);
    }
    int U(int i, int j, int k) { return object_id.U(i, j, k); }
    /* ch4/World.h:88-98: cell indices and the cell number of a position */
    int3 XtoIJK(double3 x) const {
        double3 lc = XtoL(x);
        return int3((int)lc[0], (int)lc[1], (int)lc[2]);
    }
    int XtoC(double3 x) const {
        int3 i = XtoIJK(x);
        return i[2] * (nj - 1) * (ni - 1) + i[1] * (ni - 1) + i[0];
    }
    /* ch4/World.cpp:160-199 (host): the segment's sphere crossing and a
     * diffuse direction off the sphere at x (two host rnd() draws) */
    double lineSphereIntersect(const double3 &x1, const double3 &x2);
    double3 sphereDiffuseVector(const double3 &x);

    void computeChargeDensity(std::vector<Species> &species);
    double getPE();
    void addSphere(double3 x0, double radius, double phi_sphere);
    bool inSphere(double3 x);
    void addInlet();
    bool steadyState(std::vector<Species> &species);
    /* ch4/World.h:76 */
    bool isSteadyState() const { return steady_state; }

    /* ch9/MT/World.h: the thread count is accepted and ignored on the GPU */
    void setNumThreads(int n) { num_threads = n; }
    int getNumThreads() const { return num_threads; }

    const int ni, nj, nk;
    const int3 nn;
    Field phi;
    Field rho;
    Field node_vol;
    Field3 ef;
    FieldI object_id;

    /* ---- libespic plumbing ---- */
    espic_world *handle() const { return h; }
    void push_host_edits();     /* push dirty mirrors before device work */
    void fields_written(int mask); /* bits: 1 phi, 2 rho, 4 ef, 8 object_id */

protected:
    double3 x0, dh, xm, xc;
    double dt = 0;
    double time = 0;
    int ts = -1;
    int num_ts = 0;
    int num_threads = 1;
    double3 sphere_x0{0, 0, 0};
    double sphere_rad2 = 0;
    bool steady_state = false;
    double last_mass = 0, last_mom = 0, last_en = 0;
    std::chrono::time_point<std::chrono::high_resolution_clock> time_start;
    espic_world *h = nullptr;
    void bind_fields();
};

#endif
