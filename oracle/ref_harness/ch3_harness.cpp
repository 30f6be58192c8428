/*
 * ch3_harness.cpp -- drives the reference's ch3/ver2 (flow past a sphere)
 * classes through their public API, one operation per run, for golden
 * vectors.  TEST INFRASTRUCTURE ONLY; compiled against the reference sources
 * by oracle/build_ref.py.  Usage: ref_ch3 <op> <in.kv> <out.kv>
 */
#include <chrono>
#include <cmath>
#include <iostream>
#include <random>
#include <string>
#include <vector>
#include "harness_io.h"
#define protected public
#include "World.h"
#include "Species.h"
#include "PotentialSolver.h"
#include "Source.h"
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
    if (argc != 4) { fprintf(stderr, "usage: ref_ch3 op in out\n"); return 1; }
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
    if (kv_has(in, "sphere")) {
        const std::vector<double> &s = kv_get(in, "sphere"); /* cx cy cz radius phi */
        world.addSphere(double3(s[0], s[1], s[2]), s[3], s[4]);
    }
    if (kv_has(in, "inlet")) world.addInlet();
    if (kv_has(in, "phi")) field_in(world.phi, kv_get(in, "phi"), ni, nj, nk);
    if (kv_has(in, "rho")) field_in(world.rho, kv_get(in, "rho"), ni, nj, nk);
    if (kv_has(in, "ef")) field3_in(world.ef, kv_get(in, "ef"), ni, nj, nk);

    std::vector<Species> species;
    int ns = kv_has(in, "ns") ? (int)kv_s(in, "ns") : 0;
    species.reserve(ns > 0 ? ns : 1);
    for (int s = 0; s < ns; s++) {
        std::string key = "sp" + std::to_string(s);
        const std::vector<double> &mq = kv_get(in, (key + "_mq").c_str()); /* mass charge mpw0 */
        species.push_back(Species(key, mq[0], mq[1], mq[2], world));
        if (kv_has(in, (key + "_P").c_str())) particles_in(species[s], kv_get(in, (key + "_P").c_str()));
    }

    if (op == "objects") {
        out["object_id"] = field_out(world.object_id, ni, nj, nk);
        out["phi"] = field_out(world.phi, ni, nj, nk);
    } else if (op == "push_sphere") {
        for (Species &sp : species) sp.advance();
        for (int s = 0; s < ns; s++) out["sp" + std::to_string(s) + "_P"] = particles_out(species[s]);
    } else if (op == "deposit") {
        for (int s = 0; s < ns; s++) {
            species[s].computeNumberDensity();
            out["sp" + std::to_string(s) + "_den"] = field_out(species[s].den, ni, nj, nk);
        }
    } else if (op == "gs" || op == "qn") {
        std::vector<double> phi_in = field_out(world.phi, ni, nj, nk);
        PotentialSolver solver(world, op == "gs" ? SolverType::GS : SolverType::QN,
                               (int)kv_s(in, "max_it"), kv_s(in, "tol"));
        /* the constructor's buildMatrix() ends in solveQN(); restore phi */
        field_in(world.phi, phi_in, ni, nj, nk);
        const std::vector<double> &ref = kv_get(in, "ref"); /* phi0 Te0 n0 */
        solver.setReferenceValues(ref[0], ref[1], ref[2]);
        out["conv"] = {solver.solve() ? 1.0 : 0.0};
        out["phi"] = field_out(world.phi, ni, nj, nk);
    } else if (op == "efield") {
        std::vector<double> phi_in = field_out(world.phi, ni, nj, nk);
        PotentialSolver solver(world, SolverType::QN, 1, 1.0);
        field_in(world.phi, phi_in, ni, nj, nk); /* undo the constructor's solveQN() */
        solver.computeEF();
        out["ef"] = field3_out(world.ef, ni, nj, nk);
    } else if (op == "inject_cold") {
        const std::vector<double> &src = kv_get(in, "source"); /* v_drift den */
        ColdBeamSource source(species[0], world, src[0], src[1]);
        Rnd before = rnd;
        source.sample();
        out["u"] = replay(before);
        out["sp0_P"] = particles_out(species[0]);
    } else if (op == "update_average") {
        const std::vector<double> &seq = kv_get(in, "dens"); /* m fields back to back */
        size_t nn = (size_t)ni * nj * nk;
        for (size_t m = 0; m * nn < seq.size(); m++) {
            std::vector<double> f(seq.begin() + m * nn, seq.begin() + (m + 1) * nn);
            field_in(species[0].den, f, ni, nj, nk);
            species[0].updateAverages();
        }
        out["den_ave"] = field_out(species[0].den_ave, ni, nj, nk);
    } else if (op == "steps") {
        /* the loop body of ch3/ver2/Main.cpp:50-80 without file output */
        const std::vector<double> &src = kv_get(in, "source");
        std::vector<ColdBeamSource> sources;
        sources.push_back(ColdBeamSource(species[0], world, src[0], src[1]));
        std::vector<double> phi_in = field_out(world.phi, ni, nj, nk);
        PotentialSolver solver(world, SolverType::GS, (int)kv_s(in, "max_it"), kv_s(in, "tol"));
        field_in(world.phi, phi_in, ni, nj, nk);
        const std::vector<double> &ref = kv_get(in, "ref");
        solver.setReferenceValues(ref[0], ref[1], ref[2]);
        if (kv_has(in, "initial_solve")) {
            solver.solve();
            solver.computeEF();
        }
        std::vector<double> hist, us, ucount;
        /* optional batch means of den (species 0) and phi: avg = [first ts, steps per batch, batches] */
        int a_from = 0, a_len = 0, a_nb = 0;
        if (kv_has(in, "avg")) {
            const std::vector<double> &a = kv_get(in, "avg");
            a_from = (int)a[0]; a_len = (int)a[1]; a_nb = (int)a[2];
        }
        size_t nn = (size_t)ni * nj * nk;
        std::vector<double> den_b((size_t)a_nb * nn, 0.0), phi_b((size_t)a_nb * nn, 0.0);
        while (world.advanceTime()) {
            Rnd before = rnd;
            for (ColdBeamSource &s : sources) s.sample();
            std::vector<double> u = replay(before);
            ucount.push_back((double)u.size());
            us.insert(us.end(), u.begin(), u.end());
            for (Species &sp : species) {
                sp.advance();
                sp.computeNumberDensity();
            }
            world.computeChargeDensity(species);
            solver.solve();
            solver.computeEF();
            double ss = world.steadyState(species) ? 1.0 : 0.0;
            if (ss > 0)
                for (Species &sp : species) sp.updateAverages();
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
            hist.push_back(ss);
            int ts = world.getTs();
            if (a_len > 0 && ts >= a_from && (ts - a_from) / a_len < a_nb) {
                size_t b = (size_t)((ts - a_from) / a_len) * nn;
                std::vector<double> d = field_out(species[0].den, ni, nj, nk);
                std::vector<double> p = field_out(world.phi, ni, nj, nk);
                for (size_t n = 0; n < nn; n++) {
                    den_b[b + n] += d[n] / a_len;
                    phi_b[b + n] += p[n] / a_len;
                }
            }
        }
        if (a_nb > 0) {
            out["sp0_den_batches"] = den_b;
            out["phi_batches"] = phi_b;
        }
        out["hist"] = hist;
        out["u"] = us;
        out["u_count"] = ucount;
        out["phi"] = field_out(world.phi, ni, nj, nk);
        out["ef"] = field3_out(world.ef, ni, nj, nk);
        for (int s = 0; s < ns; s++) {
            out["sp" + std::to_string(s) + "_P"] = particles_out(species[s]);
            out["sp" + std::to_string(s) + "_den"] = field_out(species[s].den, ni, nj, nk);
            out["sp" + std::to_string(s) + "_den_ave"] = field_out(species[s].den_ave, ni, nj, nk);
        }
    } else {
        fprintf(stderr, "unknown op %s\n", op.c_str());
        return 1;
    }
    kv_write(argv[3], out);
    return 0;
}
