/*
 * ch4_harness.cpp -- drives the reference's ch4 WarmBeamSource (drifting
 * isotropic thermal injector), DSMC_MEX (neutral-neutral collisions),
 * Species moment sampling, MCC_CEX (charge exchange) and the neutral push
 * with the sphere's diffuse reflection through their public API for golden
 * vectors.
 * TEST INFRASTRUCTURE ONLY; compiled against the reference sources by
 * oracle/build_ref.py.  Usage: ref_ch4 inject_warm|dsmc|moments|mcc|advance|advance_ion|ionize <in.kv> <out.kv>
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
#include "Source.h"
#include "Collisions.h"
#undef protected

int main(int argc, char **argv) {
    if (argc != 4) { fprintf(stderr, "usage: ref_ch4 op in out\n"); return 1; }
    std::string op = argv[1];
    KV in = kv_read(argv[2]), out;
    const std::vector<double> &gd = kv_get(in, "grid");
    int ni = (int)gd[0], nj = (int)gd[1], nk = (int)gd[2];
    const std::vector<double> &x0 = kv_get(in, "x0"), &xm = kv_get(in, "xm");
    World world(ni, nj, nk);
    world.setExtents(double3(x0[0], x0[1], x0[2]), double3(xm[0], xm[1], xm[2]));
    world.setTime(kv_s(in, "dt"), 1);
    rnd.mt_gen.seed((unsigned)kv_s(in, "seed"));
    if (kv_has(in, "ef")) field3_in(world.ef, kv_get(in, "ef"), ni, nj, nk);
    const std::vector<double> &mq = kv_get(in, "sp0_mq");
    Species sp("sp0", mq[0], mq[1], mq[2], world);
    if (op == "dsmc") {
        /* DSMC_MEX::apply(dt) `steps` times on the given particles; the
         * uniforms it drew are recorded by replaying the generator */
        const std::vector<double> &P = kv_get(in, "sp0_P");
        size_t n = P.size() / 7;
        for (size_t p = 0; p < n; p++)
            sp.particles.emplace_back(double3(P[p], P[n + p], P[2 * n + p]),
                                      double3(P[3 * n + p], P[4 * n + p], P[5 * n + p]), 0.0, P[6 * n + p]);
        DSMC_MEX dsmc(sp, world);
        if (kv_has(in, "sigma_cr_max")) dsmc.sigma_cr_max = kv_s(in, "sigma_cr_max");
        int steps = kv_has(in, "steps") ? (int)kv_s(in, "steps") : 1;
        std::vector<double> us, smax;
        for (int s = 0; s < steps; s++) {
            Rnd before = rnd;
            dsmc.apply(kv_s(in, "dt"));
            for (long g = 0; g < 2000000000L && !(before.mt_gen == rnd.mt_gen); g++) us.push_back(before());
            smax.push_back(dsmc.sigma_cr_max);
        }
        std::vector<double> v(7 * n);
        for (size_t p = 0; p < n; p++) {
            for (int d = 0; d < 3; d++) {
                v[d * n + p] = sp.particles[p].pos[d];
                v[(3 + d) * n + p] = sp.particles[p].vel[d];
            }
            v[6 * n + p] = sp.particles[p].mpw;
        }
        out["u"] = us;
        out["sigma_cr_max"] = smax;
        out["c"] = std::vector<double>(dsmc.c, dsmc.c + 4);
        out["sp0_P"] = v;
        kv_write(argv[3], out);
        return 0;
    }
    if (op == "moments" || op == "mcc") {
        const std::vector<double> &P = kv_get(in, "sp0_P");
        size_t n = P.size() / 7;
        for (size_t p = 0; p < n; p++)
            sp.particles.emplace_back(double3(P[p], P[n + p], P[2 * n + p]),
                                      double3(P[3 * n + p], P[4 * n + p], P[5 * n + p]), 0.0, P[6 * n + p]);
        if (op == "moments") {
            /* sampleMoments `calls` times (particles unchanged), then
             * computeGasProperties and computeMPC */
            int calls = kv_has(in, "calls") ? (int)kv_s(in, "calls") : 1;
            for (int c = 0; c < calls; c++) sp.sampleMoments();
            sp.computeGasProperties();
            sp.computeMPC();
            std::vector<double> mom;
            for (Field *f : {&sp.n_sum}) {
                std::vector<double> a = field_out(*f, ni, nj, nk);
                mom.insert(mom.end(), a.begin(), a.end());
            }
            std::vector<double> nv = field3_out(sp.nv_sum, ni, nj, nk); /* [nn][3] */
            for (int d = 0; d < 3; d++)
                for (size_t u = 0; u < nv.size() / 3; u++) mom.push_back(nv[3 * u + d]);
            for (Field *f : {&sp.nuu_sum, &sp.nvv_sum, &sp.nww_sum}) {
                std::vector<double> a = field_out(*f, ni, nj, nk);
                mom.insert(mom.end(), a.begin(), a.end());
            }
            out["mom"] = mom;
            out["vel"] = field3_out(sp.vel, ni, nj, nk);
            out["T"] = field_out(sp.T, ni, nj, nk);
            out["mpc"] = field_out(sp.mpc, ni - 1, nj - 1, nk - 1);
            kv_write(argv[3], out);
            return 0;
        }
        /* MCC_CEX(sp0 -> sp1).apply(dt) `steps` times; sp1's den and vel are
         * given; the uniforms drawn are recorded by replaying the generator */
        const std::vector<double> &mq1 = kv_get(in, "sp1_mq");
        Species tgt("sp1", mq1[0], mq1[1], mq1[2], world);
        field_in(tgt.den, kv_get(in, "sp1_den"), ni, nj, nk);
        field3_in(tgt.vel, kv_get(in, "sp1_vel"), ni, nj, nk);
        field_in(tgt.T, kv_get(in, "sp1_T"), ni, nj, nk);
        MCC_CEX mcc(sp, tgt, world);
        int steps = kv_has(in, "steps") ? (int)kv_s(in, "steps") : 1;
        std::vector<double> us;
        for (int s = 0; s < steps; s++) {
            Rnd before = rnd;
            mcc.apply(kv_s(in, "dt"));
            for (long g = 0; g < 2000000000L && !(before.mt_gen == rnd.mt_gen); g++) us.push_back(before());
        }
        std::vector<double> v(7 * n);
        for (size_t p = 0; p < n; p++) {
            for (int d = 0; d < 3; d++) {
                v[d * n + p] = sp.particles[p].pos[d];
                v[(3 + d) * n + p] = sp.particles[p].vel[d];
            }
            v[6 * n + p] = sp.particles[p].mpw;
        }
        out["u"] = us;
        out["sp0_P"] = v;
        kv_write(argv[3], out);
        return 0;
    }
    if (op == "advance") {
        /* Species::advance(sp, sp) of a neutral species `steps` times with the
         * sphere's diffuse reflection; sp0_dt: each particle's time left */
        const std::vector<double> &P = kv_get(in, "sp0_P"), &pdt = kv_get(in, "sp0_dt");
        const std::vector<double> &sph = kv_get(in, "sphere"); /* cx cy cz r phi */
        world.addSphere(double3(sph[0], sph[1], sph[2]), sph[3], sph[4]);
        size_t n = P.size() / 7;
        for (size_t p = 0; p < n; p++)
            sp.particles.emplace_back(double3(P[p], P[n + p], P[2 * n + p]),
                                      double3(P[3 * n + p], P[4 * n + p], P[5 * n + p]), pdt[p], P[6 * n + p]);
        int steps = kv_has(in, "steps") ? (int)kv_s(in, "steps") : 1;
        std::vector<double> us;
        for (int s = 0; s < steps; s++) {
            Rnd before = rnd;
            sp.advance(sp, sp);
            for (long g = 0; g < 2000000000L && !(before.mt_gen == rnd.mt_gen); g++) us.push_back(before());
        }
        n = sp.particles.size();
        std::vector<double> v(7 * n), dts(n);
        for (size_t p = 0; p < n; p++) {
            for (int d = 0; d < 3; d++) {
                v[d * n + p] = sp.particles[p].pos[d];
                v[(3 + d) * n + p] = sp.particles[p].vel[d];
            }
            v[6 * n + p] = sp.particles[p].mpw;
            dts[p] = sp.particles[p].dt;
        }
        out["u"] = us;
        out["sp0_P"] = v;
        out["sp0_dt"] = dts;
        kv_write(argv[3], out);
        return 0;
    }
    if (op == "advance_ion") {
        /* Species::advance(sp1, sp1) of a charged species sp0 `steps` times:
         * ions striking the sphere create neutrals and sputtered particles
         * in sp1 (as ch4/Main.cpp calls it) */
        const std::vector<double> &P = kv_get(in, "sp0_P"), &pdt = kv_get(in, "sp0_dt");
        const std::vector<double> &sph = kv_get(in, "sphere");
        world.addSphere(double3(sph[0], sph[1], sph[2]), sph[3], sph[4]);
        const std::vector<double> &mq1 = kv_get(in, "sp1_mq");
        Species tgt("sp1", mq1[0], mq1[1], mq1[2], world);
        size_t n = P.size() / 7;
        for (size_t p = 0; p < n; p++)
            sp.particles.emplace_back(double3(P[p], P[n + p], P[2 * n + p]),
                                      double3(P[3 * n + p], P[4 * n + p], P[5 * n + p]), pdt[p], P[6 * n + p]);
        int steps = kv_has(in, "steps") ? (int)kv_s(in, "steps") : 1;
        std::vector<double> us;
        for (int s = 0; s < steps; s++) {
            Rnd before = rnd;
            sp.advance(tgt, tgt);
            for (long g = 0; g < 2000000000L && !(before.mt_gen == rnd.mt_gen); g++) us.push_back(before());
        }
        for (Species *q : {&sp, &tgt}) {
            size_t m = q->particles.size();
            std::vector<double> v(7 * m), dts(m);
            for (size_t p = 0; p < m; p++) {
                for (int d = 0; d < 3; d++) {
                    v[d * m + p] = q->particles[p].pos[d];
                    v[(3 + d) * m + p] = q->particles[p].vel[d];
                }
                v[6 * m + p] = q->particles[p].mpw;
                dts[p] = q->particles[p].dt;
            }
            out[q == &sp ? "sp0_P" : "sp1_P"] = v;
            out[q == &sp ? "sp0_dt" : "sp1_dt"] = dts;
        }
        out["u"] = us;
        kv_write(argv[3], out);
        return 0;
    }
    if (op == "ionize") {
        /* ChemistryIonize(sp1 neutrals, sp0 ions, world, rate).apply(dt)
         * with sp1's density and the world's rho given */
        const std::vector<double> &mq1 = kv_get(in, "sp1_mq");
        Species neu("sp1", mq1[0], mq1[1], mq1[2], world);
        field_in(neu.den, kv_get(in, "sp1_den"), ni, nj, nk);
        field_in(world.rho, kv_get(in, "rho"), ni, nj, nk);
        ChemistryIonize chem(neu, sp, world, kv_s(in, "rate"));
        Rnd before = rnd;
        chem.apply(kv_s(in, "dt"));
        std::vector<double> us;
        for (long g = 0; g < 2000000000L && !(before.mt_gen == rnd.mt_gen); g++) us.push_back(before());
        size_t m = sp.particles.size();
        std::vector<double> v(7 * m), dts(m);
        for (size_t p = 0; p < m; p++) {
            for (int d = 0; d < 3; d++) {
                v[d * m + p] = sp.particles[p].pos[d];
                v[(3 + d) * m + p] = sp.particles[p].vel[d];
            }
            v[6 * m + p] = sp.particles[p].mpw;
            dts[p] = sp.particles[p].dt;
        }
        out["u"] = us;
        out["sp0_P"] = v;
        out["sp0_dt"] = dts;
        kv_write(argv[3], out);
        return 0;
    }
    if (op != "inject_warm") { fprintf(stderr, "unknown op\n"); return 1; }
    const std::vector<double> &src = kv_get(in, "source"); /* v_drift den T */
    WarmBeamSource source(sp, world, src[0], src[1], src[2]);
    Rnd before = rnd;
    source.sample();
    std::vector<double> us;
    for (long g = 0; g < 200000000L && !(before.mt_gen == rnd.mt_gen); g++) us.push_back(before());
    size_t n = sp.particles.size();
    std::vector<double> v(7 * n);
    for (size_t p = 0; p < n; p++) {
        for (int d = 0; d < 3; d++) {
            v[d * n + p] = sp.particles[p].pos[d];
            v[(3 + d) * n + p] = sp.particles[p].vel[d];
        }
        v[6 * n + p] = sp.particles[p].mpw;
    }
    out["u"] = us;
    out["sp0_P"] = v;
    kv_write(argv[3], out);
    return 0;
}
