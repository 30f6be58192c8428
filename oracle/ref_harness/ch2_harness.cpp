/*
 * ch2_harness.cpp -- drives the reference's ch2 (grounded box) classes
 * through their public API, one operation per run, for golden vectors.
 * TEST INFRASTRUCTURE ONLY; compiled against the reference sources by
 * oracle/build_ref.py.  Usage: ref_ch2 <op> <in.kv> <out.kv>
 */
#include <chrono>
#include <cmath>
#include <iostream>
#include <random>
#include <string>
#include <vector>
#include "harness_io.h"
/* The harness seeds the reference's global Rnd (a protected mt19937) and
 * replays it to record the uniforms an operation consumed. */
#define protected public
#include "World.h"
#include "Species.h"
#include "PotentialSolver.h"
#undef protected

static std::vector<double> particles_out(Species &sp) {
    size_t n = sp.particles.size();
    std::vector<double> v(7 * n);
    for (size_t p = 0; p < n; p++) {
        Particle &q = sp.particles[p];
        for (int d = 0; d < 3; d++) {
            v[d * n + p] = q.pos[d];
            v[(3 + d) * n + p] = q.vel[d];
        }
        v[6 * n + p] = q.mpw;
    }
    return v;
}

static void particles_in(Species &sp, const std::vector<double> &v) {
    size_t n = v.size() / 7;
    sp.particles.clear();
    for (size_t p = 0; p < n; p++)
        sp.particles.emplace_back(double3(v[p], v[n + p], v[2 * n + p]),
                                  double3(v[3 * n + p], v[4 * n + p], v[5 * n + p]), v[6 * n + p]);
}

static std::vector<double> replay(Rnd &before) {
    std::vector<double> us;
    for (long guard = 0; guard < 200000000L && !(before.mt_gen == rnd.mt_gen); guard++)
        us.push_back(before());
    return us;
}

int main(int argc, char **argv) {
    if (argc != 4) { fprintf(stderr, "usage: ref_ch2 op in out\n"); return 1; }
    std::string op = argv[1];
    KV in = kv_read(argv[2]), out;
    const std::vector<double> &gd = kv_get(in, "grid");
    int ni = (int)gd[0], nj = (int)gd[1], nk = (int)gd[2];
    const std::vector<double> &x0 = kv_get(in, "x0"), &xm = kv_get(in, "xm");
    World world(ni, nj, nk);
    world.setExtents(double3(x0[0], x0[1], x0[2]), double3(xm[0], xm[1], xm[2]));
    double dt = kv_has(in, "dt") ? kv_s(in, "dt") : 0.0;
    int steps = kv_has(in, "steps") ? (int)kv_s(in, "steps") : 1;
    world.setTime(dt, steps);
    if (kv_has(in, "seed")) rnd.mt_gen.seed((unsigned)kv_s(in, "seed"));
    if (kv_has(in, "phi")) field_in(world.phi, kv_get(in, "phi"), ni, nj, nk);
    if (kv_has(in, "rho")) field_in(world.rho, kv_get(in, "rho"), ni, nj, nk);
    if (kv_has(in, "ef")) field3_in(world.ef, kv_get(in, "ef"), ni, nj, nk);

    std::vector<Species> species;
    int ns = kv_has(in, "ns") ? (int)kv_s(in, "ns") : 0;
    species.reserve(ns > 0 ? ns : 1);
    for (int s = 0; s < ns; s++) {
        std::string key = "sp" + std::to_string(s);
        const std::vector<double> &mq = kv_get(in, (key + "_mq").c_str());
        species.push_back(Species(key, mq[0], mq[1], world));
        if (kv_has(in, (key + "_P").c_str())) particles_in(species[s], kv_get(in, (key + "_P").c_str()));
    }

    if (op == "node_vol") {
        out["node_vol"] = field_out(world.node_vol, ni, nj, nk);
    } else if (op == "push") {
        for (Species &sp : species) sp.advance();
        for (int s = 0; s < ns; s++) out["sp" + std::to_string(s) + "_P"] = particles_out(species[s]);
    } else if (op == "deposit") {
        for (int s = 0; s < ns; s++) {
            species[s].computeNumberDensity();
            out["sp" + std::to_string(s) + "_den"] = field_out(species[s].den, ni, nj, nk);
        }
    } else if (op == "charge") {
        for (int s = 0; s < ns; s++) {
            std::string key = "sp" + std::to_string(s) + "_den";
            field_in(species[s].den, kv_get(in, key.c_str()), ni, nj, nk);
        }
        world.computeChargeDensity(species);
        out["rho"] = field_out(world.rho, ni, nj, nk);
    } else if (op == "sor") {
        PotentialSolver solver(world, (int)kv_s(in, "max_it"), kv_s(in, "tol"));
        out["conv"] = {solver.solve() ? 1.0 : 0.0};
        out["phi"] = field_out(world.phi, ni, nj, nk);
    } else if (op == "efield") {
        PotentialSolver solver(world, 1, 1.0);
        solver.computeEF();
        out["ef"] = field3_out(world.ef, ni, nj, nk);
    } else if (op == "diag") {
        for (int s = 0; s < ns; s++) {
            double3 m = species[s].getMomentum();
            out["sp" + std::to_string(s) + "_diag"] = {species[s].getRealCount(), m[0], m[1], m[2],
                                                       species[s].getKE()};
        }
        out["pe"] = {world.getPE()};
    } else if (op == "load_box" || op == "load_qs") {
        const std::vector<double> &x1 = kv_get(in, "x1"), &x2 = kv_get(in, "x2");
        const std::vector<double> &nm = kv_get(in, "num_mp");
        Rnd before = rnd;
        if (op == "load_box")
            species[0].loadParticlesBox(double3(x1[0], x1[1], x1[2]), double3(x2[0], x2[1], x2[2]),
                                        kv_s(in, "num_den"), (int)nm[0]);
        else
            species[0].loadParticlesBoxQS(double3(x1[0], x1[1], x1[2]), double3(x2[0], x2[1], x2[2]),
                                          kv_s(in, "num_den"), int3((int)nm[0], (int)nm[1], (int)nm[2]));
        out["u"] = replay(before);
        out["sp0_P"] = particles_out(species[0]);
    } else if (op == "steps") {
        /* the loop body of ch2/Main.cpp:45-70 without file output */
        PotentialSolver solver(world, (int)kv_s(in, "max_it"), kv_s(in, "tol"));
        if (kv_has(in, "initial_solve")) {
            solver.solve();
            solver.computeEF();
        }
        std::vector<double> hist;
        while (world.advanceTime()) {
            for (Species &sp : species) {
                sp.advance();
                sp.computeNumberDensity();
            }
            world.computeChargeDensity(species);
            solver.solve();
            solver.computeEF();
            hist.push_back(world.getTs());
            for (Species &sp : species) {
                double3 m = sp.getMomentum();
                hist.push_back((double)sp.getNp());
                hist.push_back(sp.getRealCount());
                hist.push_back(m[0]);
                hist.push_back(m[1]);
                hist.push_back(m[2]);
                hist.push_back(sp.getKE());
            }
            hist.push_back(world.getPE());
        }
        out["hist"] = hist;
        out["phi"] = field_out(world.phi, ni, nj, nk);
        out["ef"] = field3_out(world.ef, ni, nj, nk);
        for (int s = 0; s < ns; s++) {
            out["sp" + std::to_string(s) + "_P"] = particles_out(species[s]);
            out["sp" + std::to_string(s) + "_den"] = field_out(species[s].den, ni, nj, nk);
        }
    } else {
        fprintf(stderr, "unknown op %s\n", op.c_str());
        return 1;
    }
    kv_write(argv[3], out);
    return 0;
}
