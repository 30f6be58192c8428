/*
 * ch9mpi_harness.cpp -- drives the particle source of the reference's ch9/MPI
 * variant (Source::sample, ch9/MPI/src/Source.cpp:5-72: fixed-speed isotropic
 * thermal velocities, v_z < 0 reflected, the fractional macroparticle count
 * carried between calls) through its public API, for golden vectors.
 * TEST INFRASTRUCTURE ONLY; compiled with the stand-in mpi.h of mpi_stub/ by
 * oracle/build_ref.py.  Usage: ref_ch9mpi sample <in.kv> <out.kv>
 *
 * The harness provides the rnd() that ch9/MPI's main program defines
 * (ch9/MPI/src/Sphere.cpp:31-38: mt19937, uniform on [0,1)), seeded from the
 * input, and records every uniform drawn.
 */
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <list>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>
#include "harness_io.h"
/* the standard headers come first: only the reference's classes are opened */
#define private public
#define protected public
#include "World.h"
#include "Field.h"
#include "Species.h"
#include "Source.h"
#undef protected
#undef private

static std::mt19937 g_gen;
static std::uniform_real_distribution<double> g_dist(0, 1.0);
static std::vector<double> g_used;
double rnd() {
    double u = g_dist(g_gen);
    g_used.push_back(u);
    return u;
}

int main(int argc, char **argv) {
    if (argc != 4) { fprintf(stderr, "usage: ref_ch9mpi op in out\n"); return 1; }
    std::string op = argv[1];
    KV in = kv_read(argv[2]), out;
    const std::vector<double> &gd = kv_get(in, "grid");
    int ni = (int)gd[0], nj = (int)gd[1], nk = (int)gd[2];
    const std::vector<double> &x0 = kv_get(in, "x0"), &dh = kv_get(in, "dh");
    World world(ni, nj, nk);
    world.setOrigin(x0[0], x0[1], x0[2]);
    world.setSpacing(dh[0], dh[1], dh[2]);
    world.setDt(kv_s(in, "dt"));
    world.mpi_k = 0;
    if (kv_has(in, "ef")) {
        const std::vector<double> &ef = kv_get(in, "ef"); /* [nn][3] in U order */
        for (int k = 0; k < nk; k++)
            for (int j = 0; j < nj; j++)
                for (int i = 0; i < ni; i++) {
                    size_t u = ((size_t)k * nj + j) * ni + i;
                    for (int d = 0; d < 3; d++) world.ef->f[d]->data[i][j][k] = ef[3 * u + d];
                }
    }
    g_gen.seed((unsigned)kv_s(in, "seed"));
    const std::vector<double> &sp = kv_get(in, "species"); /* mass, charge, spwt, capacity */
    Species species(world, "ions", sp[0], sp[1], sp[2], (int)sp[3]);
    const std::vector<double> &src = kv_get(in, "source"); /* den0, v_drift, T */
    Source source(world, species, src[0], src[1], src[2]);
    if (op != "sample") { fprintf(stderr, "unknown op %s\n", op.c_str()); return 1; }
    int calls = (int)kv_s(in, "calls");
    std::vector<double> counts, rems, used;
    for (int c = 0; c < calls; c++) {
        int before = species.np;
        size_t u0 = g_used.size();
        source.sample();
        counts.push_back(species.np - before);
        rems.push_back(source.num_rem);
        used.push_back((double)(g_used.size() - u0));
    }
    int n = species.np;
    std::vector<double> P(7 * (size_t)n);
    for (int p = 0; p < n; p++) {
        for (int d = 0; d < 3; d++) {
            P[d * (size_t)n + p] = species.particles[p].pos[d];
            P[(3 + d) * (size_t)n + p] = species.particles[p].vel[d];
        }
        P[6 * (size_t)n + p] = species.spwt;
    }
    out["P"] = P;
    out["counts"] = counts;
    out["rem"] = rems;
    out["used"] = used;
    out["u"] = g_used;
    out["v_th"] = {source.v_th};
    kv_write(argv[3], out);
    return 0;
}
