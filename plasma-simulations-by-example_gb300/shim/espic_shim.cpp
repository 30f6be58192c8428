/*
 * espic_shim.cpp -- the drop-in World / Species / PotentialSolver / sources /
 * Output classes, implemented on the libespic C-ABI (include/espic.h).
 * Compile the reference's unchanged Main.cpp against the headers of this
 * directory, add this file, and link -lespic.
 *
 * Environment knobs (no reference counterpart): ESPIC_CAPACITY (particles
 * per species kept on the GPU, default 16M), ESPIC_FORM=mixed (store
 * species with a default weight in the mixed form), ESPIC_SEED (Philox key).
 */
#include <cmath>
#include <deque>
#include <thread>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>

#include "Collisions.h"
#include "Output.h"
#include "PotentialSolver.h"
#include "Source.h"
#include "Species.h"
#include "World.h"
#include "espic.h"

Rnd rnd;

/* set once the program uses the ch4 species API: Output::fields then writes
 * ch4's file layout (ch4/Output.cpp:11-119) */
static bool g_ch4_layout = false;

static void ck(int rc, const char *what) {
    if (rc >= 0) return;
    char msg[512];
    espic_last_error(msg, sizeof msg);
    throw std::runtime_error(std::string(what) + ": " + msg);
}

static int64_t env_int(const char *name, int64_t def) {
    const char *v = getenv(name);
    return v && *v ? atoll(v) : def;
}

/* ------------------------------------------------------------------ World */
World::World(int ni, int nj, int nk)
    : ni{ni}, nj{nj}, nk{nk}, nn{ni, nj, nk}, phi(ni, nj, nk), rho(ni, nj, nk), node_vol(ni, nj, nk),
      ef(ni, nj, nk), object_id(ni, nj, nk) {
    time_start = std::chrono::high_resolution_clock::now();
}

static void join_output_writers();

World::~World() {
    join_output_writers(); /* files still being written read this world's snapshots */
    if (h) espic_world_destroy(h);
}

void World::setExtents(const double3 _x0, const double3 _xm) {
    x0 = _x0;
    xm = _xm;
    for (int i = 0; i < 3; i++) dh[i] = (xm(i) - x0(i)) / (nn(i) - 1);
    xc = 0.5 * (x0 + xm);
    if (h) {
        espic_world_destroy(h);
        h = nullptr;
    }
    double a[3] = {x0(0), x0(1), x0(2)}, b[3] = {xm(0), xm(1), xm(2)};
    ck(espic_world_create(ni, nj, nk, a, b, &h), "espic_world_create");
    int64_t seed = env_int("ESPIC_SEED", 0);
    if (seed) espic_world_set_seed(h, (uint64_t)seed);
    if (dt > 0) espic_world_set_time(h, dt, num_ts);
    bind_fields();
    fields_written(1 | 2 | 4 | 8 | 16);
}

void World::bind_fields() {
    espic_world *hh = h;
    int64_t n = (int64_t)ni * nj * nk;
    auto bind_d = [hh, n](Field &f, int id) {
        f.bind([hh, n, id](void *dst) { ck(espic_field_read(hh, id, 0, (double *)dst, n), "espic_field_read"); },
               [hh, n, id](const void *src) {
                   ck(espic_field_write(hh, id, 0, (const double *)src, n), "espic_field_write");
               });
    };
    bind_d(phi, ESPIC_FIELD_PHI);
    bind_d(rho, ESPIC_FIELD_RHO);
    bind_d(node_vol, ESPIC_FIELD_NODE_VOL);
    ef.bind([hh, n](void *dst) { ck(espic_field_read(hh, ESPIC_FIELD_EF, 0, (double *)dst, 3 * n), "read ef"); },
            [hh, n](const void *src) {
                ck(espic_field_write(hh, ESPIC_FIELD_EF, 0, (const double *)src, 3 * n), "write ef");
            });
    object_id.bind(
        [hh, n](void *dst) {
            std::vector<double> tmp(n);
            ck(espic_field_read(hh, ESPIC_FIELD_OBJECT_ID, 0, tmp.data(), n), "read object_id");
            int *o = (int *)dst;
            for (int64_t u = 0; u < n; u++) o[u] = (int)tmp[u];
        },
        [hh, n](const void *src) {
            std::vector<double> tmp(n);
            const int *o = (const int *)src;
            for (int64_t u = 0; u < n; u++) tmp[u] = o[u];
            ck(espic_field_write(hh, ESPIC_FIELD_OBJECT_ID, 0, tmp.data(), n), "write object_id");
        });
}

void World::push_host_edits() {
    phi.push();
    rho.push();
    node_vol.push();
    ef.push();
    object_id.push();
}

void World::fields_written(int mask) {
    if (mask & 1) phi.device_written();
    if (mask & 2) rho.device_written();
    if (mask & 4) ef.device_written();
    if (mask & 8) object_id.device_written();
    if (mask & 16) node_vol.device_written();
}

double World::getWallTime() {
    auto now = std::chrono::high_resolution_clock::now();
    std::chrono::duration<double> d = now - time_start;
    return d.count();
}

void World::setTime(double dt_, int num_ts_) {
    dt = dt_;
    num_ts = num_ts_;
    if (h) ck(espic_world_set_time(h, dt, num_ts), "espic_world_set_time");
}

bool World::advanceTime() {
    time += dt;
    ts++;
    if (h) espic_world_advance_time(h);
    return ts <= num_ts;
}

void World::computeChargeDensity(std::vector<Species> &species) {
    for (Species &sp : species) {
        sp.settle();
        sp.den.push();
    }
    push_host_edits();
    ck(espic_charge_density(h), "espic_charge_density");
    fields_written(2);
}

double World::getPE() {
    push_host_edits();
    double pe = 0;
    ck(espic_potential_energy(h, &pe), "espic_potential_energy");
    return pe;
}

void World::addSphere(double3 c, double radius, double phi_sphere) {
    sphere_x0 = c;
    sphere_rad2 = radius * radius;
    push_host_edits();
    double cc[3] = {c(0), c(1), c(2)};
    ck(espic_world_add_sphere(h, cc, radius, phi_sphere), "espic_world_add_sphere");
    fields_written(1 | 8);
}

bool World::inSphere(double3 x) {
    double3 r = x - sphere_x0;
    double r_mag2 = (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    return r_mag2 <= sphere_rad2;
}

void World::addInlet() {
    push_host_edits();
    ck(espic_world_add_inlet(h), "espic_world_add_inlet");
    fields_written(1 | 8);
}

/* World::steadyState, ch3/ver2/World.cpp:129-158 */
bool World::steadyState(std::vector<Species> &species) {
    if (steady_state) return true;
    double tot_mass = 0, tot_mom = 0, tot_en = getPE();
    for (Species &sp : species) {
        tot_mass += sp.getRealCount();
        double3 mom = sp.getMomentum();
        tot_mom += std::abs(mom[2]);
        tot_en += sp.getKE();
    }
    const double tol = 1e-3;
    if (std::abs((tot_mass - last_mass) / tot_mass) < tol && std::abs((tot_mom - last_mom) / tot_mom) < tol &&
        std::abs((tot_en - last_en) / tot_en) < tol) {
        steady_state = true;
        std::cout << "Steady state reached at time step " << ts << std::endl;
    }
    last_mass = tot_mass;
    last_mom = tot_mom;
    last_en = tot_en;
    return steady_state;
}

/* World::lineSphereIntersect, ch4/World.cpp:160-182 */
double World::lineSphereIntersect(const double3 &x1, const double3 &x2) {
    double3 B = x2 - x1;
    double3 A = x1 - sphere_x0;
    double a = dot(B, B);
    double b = 2 * dot(A, B);
    double c = dot(A, A) - sphere_rad2;
    double det = b * b - 4 * a * c;
    if (det < 0) return 0.5;
    double tp = (-b + sqrt(det)) / (2 * a);
    if (tp < 0 || tp > 1.0) {
        tp = (-b - sqrt(det)) / (2 * a);
        if (tp < 0 || tp > 1.0) {
            std::cerr << "Failed to find a line-sphere intersection!" << std::endl;
            tp = 0.5;
        }
    }
    return tp;
}

/* World::sphereDiffuseVector, ch4/World.cpp:185-199 */
double3 World::sphereDiffuseVector(const double3 &x) {
    double sin_theta = rnd();
    double cos_theta = sqrt(1 - sin_theta * sin_theta);
    double psi = 2 * Const::PI * rnd();
    double3 n = unit(x - sphere_x0);
    double3 t1;
    if (dot(n, double3(1, 0, 0)) != 0)
        t1 = cross(n, double3(1, 0, 0));
    else
        t1 = cross(n, double3(0, 1, 0));
    double3 t2 = cross(n, t1);
    return sin_theta * cos(psi) * t1 + sin_theta * sin(psi) * t2 + cos_theta * n;
}

/* ---------------------------------------------------------------- Species */
std::vector<Particle> &ParticleVector::host() {
    if (!host_valid) {
        owner->pull_particles(v);
        host_valid = true;
        host_dirty = false;
    }
    return v;
}

Species::Species(std::string name, double mass, double charge, World &world)
    : name(name), mass(mass), charge(charge), mpw0(0), den(world.ni, world.nj, world.nk),
      den_ave(world.ni, world.nj, world.nk), T(world.ni, world.nj, world.nk), vel(world.ni, world.nj, world.nk),
      mpc(world.ni - 1, world.nj - 1, world.nk - 1), world(world) {
    create(ESPIC_WALLS_REFLECT);
}

Species::Species(std::string name, double mass, double charge, double mpw0, World &world)
    : name(name), mass(mass), charge(charge), mpw0(mpw0), den(world.ni, world.nj, world.nk),
      den_ave(world.ni, world.nj, world.nk), T(world.ni, world.nj, world.nk), vel(world.ni, world.nj, world.nk),
      mpc(world.ni - 1, world.nj - 1, world.nk - 1), world(world) {
    create(ESPIC_WALLS_ABSORB);
}

Species::Species(Species &&o) noexcept
    : name(o.name), mass(o.mass), charge(o.charge), mpw0(o.mpw0), particles(std::move(o.particles)),
      den(std::move(o.den)), den_ave(std::move(o.den_ave)), T(std::move(o.T)), vel(std::move(o.vel)),
      mpc(std::move(o.mpc)), world(o.world), sid(o.sid), push_pending(o.push_pending), diag_valid(o.diag_valid) {
    particles.owner = this;
    memcpy(diag, o.diag, sizeof diag);
    o.sid = -1;
}

void Species::create(int walls) {
    if (!world.handle()) throw std::runtime_error("Species: call World::setExtents first");
    int64_t cap = env_int("ESPIC_CAPACITY", 16 << 20);
    const char *f = getenv("ESPIC_FORM");
    int form = (f && !strcmp(f, "mixed") && mpw0 > 0) ? ESPIC_FORM_MIXED : ESPIC_FORM_FP64;
    ck(espic_species_create(world.handle(), mass, charge, mpw0, cap, form, walls, 0.0, &sid),
       "espic_species_create");
    particles.owner = this;
    particles.host_valid = true;
    bind_fields();
}

void Species::bind_fields() {
    espic_world *hh = world.handle();
    int64_t n = (int64_t)world.ni * world.nj * world.nk;
    int s = sid;
    den.bind([hh, n, s](void *d) { ck(espic_field_read(hh, ESPIC_FIELD_DEN, s, (double *)d, n), "read den"); },
             [hh, n, s](const void *d) {
                 ck(espic_field_write(hh, ESPIC_FIELD_DEN, s, (const double *)d, n), "write den");
             });
    den_ave.bind(
        [hh, n, s](void *d) { ck(espic_field_read(hh, ESPIC_FIELD_DEN_AVE, s, (double *)d, n), "read den_ave"); },
        [hh, n, s](const void *d) {
            ck(espic_field_write(hh, ESPIC_FIELD_DEN_AVE, s, (const double *)d, n), "write den_ave");
        });
    /* ch4 fields: the device copies exist once first used (float64 form) */
    T.bind([hh, n, s](void *d) { ck(espic_field_read(hh, ESPIC_FIELD_TEMP, s, (double *)d, n), "read T"); },
           [hh, n, s](const void *d) { ck(espic_field_write(hh, ESPIC_FIELD_TEMP, s, (const double *)d, n), "write T"); });
    vel.bind([hh, n, s](void *d) { ck(espic_field_read(hh, ESPIC_FIELD_VEL, s, (double *)d, 3 * n), "read vel"); },
             [hh, n, s](const void *d) {
                 ck(espic_field_write(hh, ESPIC_FIELD_VEL, s, (const double *)d, 3 * n), "write vel");
             });
    int64_t nc = (int64_t)(world.ni - 1) * (world.nj - 1) * (world.nk - 1);
    mpc.bind([hh, nc, s](void *d) { ck(espic_field_read(hh, ESPIC_FIELD_MPC, s, (double *)d, nc), "read mpc"); },
             [hh, nc, s](const void *d) {
                 ck(espic_field_write(hh, ESPIC_FIELD_MPC, s, (const double *)d, nc), "write mpc");
             });
}

void Species::particles_changed() {
    particles.host_valid = false;
    diag_valid = false;
}

/* run a pending push and send host edits of the particle mirror */
void Species::settle() {
    espic_world *hh = world.handle();
    if (push_pending) {
        world.push_host_edits();
        ck(espic_push(hh, sid, 0), "espic_push");
        push_pending = false;
        particles.host_valid = false;
        diag_valid = false;
    }
    if (particles.host_dirty) {
        std::vector<Particle> &v = particles.v;
        int64_t n = (int64_t)v.size();
        std::vector<double> P(7 * (n > 0 ? n : 1));
        for (int64_t p = 0; p < n; p++) {
            for (int d = 0; d < 3; d++) {
                P[d * n + p] = v[p].pos[d];
                P[(3 + d) * n + p] = v[p].vel[d];
            }
            P[6 * n + p] = v[p].mpw;
        }
        ck(espic_species_set(hh, sid, P.data(), n, n), "espic_species_set");
        particles.host_dirty = false;
        diag_valid = false;
    }
}

void Species::pull_particles(std::vector<Particle> &out) {
    if (push_pending) settle();
    int64_t n = 0;
    ck(espic_species_count(world.handle(), sid, &n), "espic_species_count");
    std::vector<double> P(7 * (n > 0 ? n : 1));
    ck(espic_species_get(world.handle(), sid, P.data(), n, n, &n), "espic_species_get");
    out.clear();
    out.reserve(n);
    for (int64_t p = 0; p < n; p++)
        out.emplace_back(double3(P[p], P[n + p], P[2 * n + p]), double3(P[3 * n + p], P[4 * n + p], P[5 * n + p]),
                         P[6 * n + p]);
}

size_t Species::getNp() {
    settle();
    int64_t n = 0;
    ck(espic_species_count(world.handle(), sid, &n), "espic_species_count");
    return (size_t)n;
}

void Species::refresh_diag() {
    settle();
    if (!diag_valid) {
        ck(espic_species_diag(world.handle(), sid, diag), "espic_species_diag");
        diag_valid = true;
    }
}

double Species::getRealCount() {
    refresh_diag();
    return diag[0];
}

double3 Species::getMomentum() {
    refresh_diag();
    return double3(diag[1], diag[2], diag[3]);
}

double Species::getKE() {
    refresh_diag();
    return diag[4];
}

void Species::advance() {
    settle();
    push_pending = true; /* fused with the next computeNumberDensity */
    particles.host_valid = false;
    diag_valid = false;
}

void Species::computeNumberDensity() {
    espic_world *hh = world.handle();
    den.push();
    if (push_pending) {
        world.push_host_edits();
        ck(espic_push(hh, sid, 1), "espic_push");
        push_pending = false;
    } else {
        settle();
        ck(espic_deposit(hh, sid), "espic_deposit");
    }
    den.device_written();
}

void Species::addParticle(double3 pos, double3 vel, double mpwt) {
    settle();
    world.push_host_edits();
    double p[3] = {pos[0], pos[1], pos[2]}, v[3] = {vel[0], vel[1], vel[2]};
    ck(espic_species_add(world.handle(), sid, p, v, &mpwt, 1), "espic_species_add");
    particles.host_valid = false;
    diag_valid = false;
}

void Species::loadParticlesBox(double3 x1, double3 x2, double num_den, int num_mp) {
    settle();
    world.push_host_edits();
    double a[3] = {x1[0], x1[1], x1[2]}, b[3] = {x2[0], x2[1], x2[2]};
    ck(espic_species_load_box(world.handle(), sid, a, b, num_den, num_mp, nullptr), "espic_species_load_box");
    particles.host_valid = false;
    diag_valid = false;
}

void Species::loadParticlesBoxQS(double3 x1, double3 x2, double num_den, int3 num_mp) {
    settle();
    world.push_host_edits();
    double a[3] = {x1[0], x1[1], x1[2]}, b[3] = {x2[0], x2[1], x2[2]};
    int nm[3] = {num_mp[0], num_mp[1], num_mp[2]};
    ck(espic_species_load_box_qs(world.handle(), sid, a, b, num_den, nm), "espic_species_load_box_qs");
    particles.host_valid = false;
    diag_valid = false;
}

void Species::updateAverages() {
    den.push();
    den_ave.push();
    ck(espic_update_average(world.handle(), sid), "espic_update_average");
    den_ave.device_written();
}

/* ch4 Species::advance(neutrals, spherium), ch4/Species.cpp:8-100, on the
 * GPU: the neutral branch (diffuse reflection at the sphere) and the ion
 * branch (ions striking the sphere are removed and add neutrals and
 * sputtered particles to the two targets) */
void Species::advance(Species &neutrals, Species &spherium) {
    g_ch4_layout = true;
    settle();
    world.push_host_edits();
    if (charge == 0) {
        ck(espic_advance_ch4(world.handle(), sid, nullptr, nullptr, 0, nullptr, nullptr), "espic_advance_ch4");
    } else {
        neutrals.settle();
        spherium.settle();
        ck(espic_advance_ch4_ions(world.handle(), sid, neutrals.id(), spherium.id(), nullptr, nullptr, 0, nullptr,
                                  nullptr),
           "espic_advance_ch4_ions");
        neutrals.particles_changed();
        spherium.particles_changed();
    }
    particles_changed();
}

/* Species::sampleMoments / computeGasProperties / computeMPC / clearSamples,
 * ch4/Species.cpp:191-240 */
void Species::sampleMoments() {
    g_ch4_layout = true;
    settle();
    ck(espic_sample_moments(world.handle(), sid), "espic_sample_moments");
}

void Species::computeGasProperties() {
    g_ch4_layout = true;
    T.push();
    vel.push();
    ck(espic_gas_properties(world.handle(), sid), "espic_gas_properties");
    T.device_written();
    vel.device_written();
}

void Species::computeMPC() {
    g_ch4_layout = true;
    settle();
    mpc.push();
    ck(espic_compute_mpc(world.handle(), sid), "espic_compute_mpc");
    mpc.device_written();
}

void Species::clearSamples() { ck(espic_clear_samples(world.handle(), sid), "espic_clear_samples"); }

/* ------------------------------------------------------------ Collisions */
void MCC_CEX::apply(double dt) {
    g_ch4_layout = true;
    source.settle();
    target.settle();
    target.den.push();
    target.vel.push();
    world.push_host_edits();
    ck(espic_mcc_cex(world.handle(), source.id(), target.id(), dt, nullptr, 0, nullptr, nullptr), "espic_mcc_cex");
    source.particles_changed();
}

DSMC_MEX::DSMC_MEX(Species &species, World &world) : species{species}, world{world} {
    g_ch4_layout = true;
    ck(espic_dsmc_enable(world.handle(), species.id(), nullptr, 1e-14), "espic_dsmc_enable");
}

void DSMC_MEX::apply(double dt) {
    species.settle();
    ck(espic_dsmc_apply(world.handle(), species.id(), dt, nullptr, 0, nullptr), "espic_dsmc_apply");
    species.particles_changed();
}

double DSMC_MEX::sigmaCrMax() {
    double s = 0;
    ck(espic_dsmc_status(world.handle(), species.id(), &s, nullptr, nullptr), "espic_dsmc_status");
    return s;
}

/* ChemistryIonize::apply, ch4/Collisions.cpp:10-31: the neutrals' den and
 * the world's rho (host edits pushed first) at each cell centre */
void ChemistryIonize::apply(double dt) {
    g_ch4_layout = true;
    ions.settle();
    neutrals.den.push();
    world.push_host_edits();
    ck(espic_chemistry_ionize(world.handle(), neutrals.id(), ions.id(), rate, dt, nullptr, 0, nullptr, nullptr),
       "espic_chemistry_ionize");
    ions.particles_changed();
}

/* Species::sampleVth / sampleIsotropicVel, ch4/Species.cpp:149-175 (host) */
double Species::sampleVth(double T) {
    double v_th = sqrt(2 * Const::K * T / mass);
    double v1 = v_th * (rnd() + rnd() + rnd() - 1.5);
    double v2 = v_th * (rnd() + rnd() + rnd() - 1.5);
    double v3 = v_th * (rnd() + rnd() + rnd() - 1.5);
    return 3 / sqrt(2 + 2 + 2) * sqrt(v1 * v1 + v2 * v2 + v3 * v3);
}

double3 Species::sampleIsotropicVel(double T) {
    double theta = 2 * Const::PI * rnd();
    double r = -1.0 + 2 * rnd();
    double a = sqrt(1 - r * r);
    double3 d;
    d[0] = r;
    d[1] = cos(theta) * a;
    d[2] = sin(theta) * a;
    double v_th = sampleVth(T);
    return v_th * d;
}

/* ---------------------------------------------------------- PotentialSolver */
PotentialSolver::PotentialSolver(World &world, int max_it, double tol)
    : world(world), kind(ESPIC_SOLVER_SOR), max_solver_it(max_it), tolerance(tol) {}

PotentialSolver::PotentialSolver(World &world, SolverType type, int max_it, double tol)
    : world(world), kind(ESPIC_SOLVER_GS), max_solver_it(max_it), tolerance(tol) {
    switch (type) {
        case GS:
        case GSCUDA: kind = ESPIC_SOLVER_GS; break;
        case PCG: kind = ESPIC_SOLVER_PCG; break;
        case QN: kind = ESPIC_SOLVER_QN; break;
    }
    buildMatrix();
}

void PotentialSolver::configure() {
    espic_world *h = world.handle();
    ck(espic_solver_set(h, kind, (int)max_solver_it, tolerance), "espic_solver_set");
    ck(espic_solver_set_reference(h, phi0, Te0, n0), "espic_solver_set_reference");
    if (kind == ESPIC_SOLVER_PCG)
        ck(espic_solver_set_newton(h, 20, 1e-3, (int)max_solver_it, 1e-6, 0), "espic_solver_set_newton");
}

/* the matrix is applied matrix-free on the GPU; like the reference's
 * buildMatrix (ch3/ver2/PotentialSolver.cpp:146-201) this ends in solveQN */
void PotentialSolver::buildMatrix() {
    int keep = kind;
    kind = ESPIC_SOLVER_QN;
    solve();
    kind = keep;
}

bool PotentialSolver::solve() {
    world.push_host_edits();
    configure();
    int it = 0, inner = 0;
    double res = 0;
    int rc = espic_solve(world.handle(), &it, &inner, &res);
    ck(rc, "espic_solve");
    world.fields_written(1);
    if (rc == ESPIC_NOT_CONVERGED) {
        if (kind == ESPIC_SOLVER_PCG)
            std::cout << "NR+PCG failed to converge, norm = " << res << std::endl;
        else
            std::cerr << "GS failed to converge, L2=" << res << std::endl;
    }
    return rc == ESPIC_OK;
}

void PotentialSolver::computeEF() {
    world.push_host_edits();
    ck(espic_efield(world.handle()), "espic_efield");
    world.fields_written(4);
}

/* ------------------------------------------------------------------ sources */
static void sample_source(World &world, Species &sp, int &src, double v_drift, double den, double T) {
    if (src < 0) ck(espic_source_create(world.handle(), sp.id(), v_drift, den, T, &src), "espic_source_create");
    sp.settle();
    world.push_host_edits();
    ck(espic_source_sample(world.handle(), src), "espic_source_sample");
    sp.particles.host_valid = false;
    sp.particles.host_dirty = false;
}

void ColdBeamSource::sample() { sample_source(world, sp, src, v_drift, den, 0.0); }

void WarmBeamSource::sample() { sample_source(world, sp, src, v_drift, den, T); }

/* ------------------------------------------------------------------ Output */
namespace Output {
std::ofstream f_diag;
}

/* Output::fields, ch3/ver2/Output.cpp:12-79: VTK ImageData, ASCII.  The
 * fields are packed on the GPU and copied to pinned memory behind the step
 * (espic_snapshot_begin); a writer thread formats them with the same stream
 * output as the reference, so the caller's loop goes on at once.  At most
 * two files are in progress; ESPIC_OUTPUT_SYNC=1 writes inline instead. */
namespace {

struct FieldsJob {
    std::string name;
    double x0[3], dh[3];
    int ni, nj, nk;
    std::vector<std::string> species;
    int64_t ticket;
    espic_world *h;
};

/* one Field_ in the layout of its operator<<: k outer, j, i inner, a space
 * after every value, a newline after every k plane */
template <typename T>
void write_scalar(std::ostream &out, const double *v, int ni, int nj, int nk) {
    for (int k = 0; k < nk; k++, out << "\n")
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) out << (T)v[((size_t)k * nj + j) * ni + i] << " ";
}

void write_vector(std::ostream &out, const double *v, int ni, int nj, int nk) {
    for (int k = 0; k < nk; k++, out << "\n")
        for (int j = 0; j < nj; j++)
            for (int i = 0; i < ni; i++) {
                const double *e = v + 3 * (((size_t)k * nj + j) * ni + i);
                out << e[0] << " " << e[1] << " " << e[2] << " ";
            }
}

void write_fields(const FieldsJob &J, const double *snap) {
    std::ofstream out(J.name);
    if (!out.is_open()) {
        std::cerr << "Could not open " << J.name << std::endl;
        return;
    }
    const size_t nn = (size_t)J.ni * J.nj * J.nk;
    const size_t ns = J.species.size();
    out << "<VTKFile type=\"ImageData\">\n";
    out << "<ImageData Origin=\"" << J.x0[0] << " " << J.x0[1] << " " << J.x0[2] << "\" ";
    out << "Spacing=\"" << J.dh[0] << " " << J.dh[1] << " " << J.dh[2] << "\" ";
    out << "WholeExtent=\"0 " << J.ni - 1 << " 0 " << J.nj - 1 << " 0 " << J.nk - 1 << "\">\n";
    out << "<PointData>\n";
    auto array = [&out](const std::string &nm, int comps, const char *type) {
        out << "<DataArray Name=\"" << nm << "\" NumberOfComponents=\"" << comps << "\" format=\"ascii\" type=\""
            << type << "\">\n";
    };
    array("object_id", 1, "Int32");
    write_scalar<int>(out, snap, J.ni, J.nj, J.nk);
    out << "</DataArray>\n";
    array("NodeVol", 1, "Float64");
    write_scalar<double>(out, snap + nn, J.ni, J.nj, J.nk);
    out << "</DataArray>\n";
    array("phi", 1, "Float64");
    write_scalar<double>(out, snap + 2 * nn, J.ni, J.nj, J.nk);
    out << "</DataArray>\n";
    array("rho", 1, "Float64");
    write_scalar<double>(out, snap + 3 * nn, J.ni, J.nj, J.nk);
    out << "</DataArray>\n";
    for (size_t s = 0; s < ns; s++) {
        array("nd." + J.species[s], 1, "Float64");
        write_scalar<double>(out, snap + (4 + s) * nn, J.ni, J.nj, J.nk);
        out << "</DataArray>\n";
    }
    for (size_t s = 0; s < ns; s++) {
        array("nd-ave." + J.species[s], 1, "Float64");
        write_scalar<double>(out, snap + (4 + ns + s) * nn, J.ni, J.nj, J.nk);
        out << "</DataArray>\n";
    }
    array("ef", 3, "Float64");
    write_vector(out, snap + (4 + 2 * ns) * nn, J.ni, J.nj, J.nk);
    out << "</DataArray>\n";
    out << "</PointData>\n</ImageData>\n</VTKFile>\n";
}

/* writer threads of the files in progress, oldest first; joined when a
 * third file starts and at exit */
struct Writers {
    std::deque<std::thread> q;
    void join_all() {
        while (!q.empty()) {
            q.front().join();
            q.pop_front();
        }
    }
    ~Writers() { join_all(); }
} writers;

}  // namespace

static void join_output_writers() { writers.join_all(); }

namespace {

void fields_sync(World &world, std::vector<Species> &species) {
    std::stringstream name;
    name << "results/fields_" << std::setfill('0') << std::setw(5) << world.getTs() << ".vti";
    std::ofstream out(name.str());
    if (!out.is_open()) {
        std::cerr << "Could not open " << name.str() << std::endl;
        return;
    }
    double3 x0 = world.getX0(), dh = world.getDh();
    out << "<VTKFile type=\"ImageData\">\n";
    out << "<ImageData Origin=\"" << x0[0] << " " << x0[1] << " " << x0[2] << "\" ";
    out << "Spacing=\"" << dh[0] << " " << dh[1] << " " << dh[2] << "\" ";
    out << "WholeExtent=\"0 " << world.ni - 1 << " 0 " << world.nj - 1 << " 0 " << world.nk - 1 << "\">\n";
    out << "<PointData>\n";
    auto array = [&out](const std::string &nm, int comps, const char *type) {
        out << "<DataArray Name=\"" << nm << "\" NumberOfComponents=\"" << comps << "\" format=\"ascii\" type=\""
            << type << "\">\n";
    };
    array("object_id", 1, "Int32");
    out << world.object_id << "</DataArray>\n";
    array("NodeVol", 1, "Float64");
    out << world.node_vol << "</DataArray>\n";
    array("phi", 1, "Float64");
    out << world.phi << "</DataArray>\n";
    array("rho", 1, "Float64");
    out << world.rho << "</DataArray>\n";
    for (Species &sp : species) {
        array("nd." + sp.name, 1, "Float64");
        out << sp.den << "</DataArray>\n";
    }
    for (Species &sp : species) {
        array("nd-ave." + sp.name, 1, "Float64");
        out << sp.den_ave << "</DataArray>\n";
    }
    array("ef", 3, "Float64");
    out << world.ef << "</DataArray>\n";
    out << "</PointData>\n</ImageData>\n</VTKFile>\n";
}

/* ch4's layout (ch4/Output.cpp:11-119): gas properties first, the stream
 * velocity and temperature of every species among the node data, the
 * macroparticles per cell as cell data, and the samples cleared until the
 * steady state */
void fields_ch4(World &world, std::vector<Species> &species) {
    for (Species &sp : species) sp.computeGasProperties();
    std::stringstream name;
    name << "results/fields_" << std::setfill('0') << std::setw(5) << world.getTs() << ".vti";
    std::ofstream out(name.str());
    if (!out.is_open()) {
        std::cerr << "Could not open " << name.str() << std::endl;
        return;
    }
    double3 x0 = world.getX0(), dh = world.getDh();
    out << "<VTKFile type=\"ImageData\">\n";
    out << "<ImageData Origin=\"" << x0[0] << " " << x0[1] << " " << x0[2] << "\" ";
    out << "Spacing=\"" << dh[0] << " " << dh[1] << " " << dh[2] << "\" ";
    out << "WholeExtent=\"0 " << world.ni - 1 << " 0 " << world.nj - 1 << " 0 " << world.nk - 1 << "\">\n";
    out << "<PointData>\n";
    auto array = [&out](const std::string &nm, int comps, const char *type) {
        out << "<DataArray Name=\"" << nm << "\" NumberOfComponents=\"" << comps << "\" format=\"ascii\" type=\""
            << type << "\">\n";
    };
    array("object_id", 1, "Int32");
    out << world.object_id << "</DataArray>\n";
    array("NodeVol", 1, "Float64");
    out << world.node_vol << "</DataArray>\n";
    array("phi", 1, "Float64");
    out << world.phi << "</DataArray>\n";
    array("rho", 1, "Float64");
    out << world.rho << "</DataArray>\n";
    for (Species &sp : species) {
        array("nd." + sp.name, 1, "Float64");
        out << sp.den << "</DataArray>\n";
    }
    for (Species &sp : species) {
        array("nd-ave." + sp.name, 1, "Float64");
        out << sp.den_ave << "</DataArray>\n";
    }
    for (Species &sp : species) {
        array("vel." + sp.name, 3, "Float64");
        out << sp.vel << "</DataArray>\n";
    }
    for (Species &sp : species) {
        array("T." + sp.name, 1, "Float64");
        out << sp.T << "</DataArray>\n";
    }
    array("ef", 3, "Float64");
    out << world.ef << "</DataArray>\n";
    out << "</PointData>\n";
    out << "<CellData>\n";
    for (Species &sp : species) {
        array("mpc." + sp.name, 1, "Float64");
        out << sp.mpc << "</DataArray>\n";
    }
    out << "</CellData>\n";
    out << "</ImageData>\n</VTKFile>\n";
    out.close();
    if (!world.isSteadyState())
        for (Species &sp : species) sp.clearSamples();
}

}  // namespace

void Output::fields(World &world, std::vector<Species> &species) {
    if (g_ch4_layout) {
        fields_ch4(world, species);
        return;
    }
    const char *sync = std::getenv("ESPIC_OUTPUT_SYNC");
    if (sync && sync[0] == '1') {
        fields_sync(world, species);
        return;
    }
    /* host edits reach the device before the snapshot reads it */
    world.phi.push();
    world.rho.push();
    world.ef.push();
    for (Species &sp : species) {
        sp.den.push();
        sp.den_ave.push();
    }
    while (writers.q.size() >= 2) {
        writers.q.front().join();
        writers.q.pop_front();
    }
    FieldsJob J;
    std::stringstream name;
    name << "results/fields_" << std::setfill('0') << std::setw(5) << world.getTs() << ".vti";
    J.name = name.str();
    double3 x0 = world.getX0(), dh = world.getDh();
    for (int d = 0; d < 3; d++) {
        J.x0[d] = x0[d];
        J.dh[d] = dh[d];
    }
    J.ni = world.ni;
    J.nj = world.nj;
    J.nk = world.nk;
    for (Species &sp : species) J.species.push_back(sp.name);
    J.h = world.handle();
    ck(espic_snapshot_begin(J.h, &J.ticket), "Output::fields");
    writers.q.emplace_back([J]() {
        const double *snap = nullptr;
        int64_t count = 0;
        if (espic_snapshot_wait(J.h, J.ticket, &snap, &count) != ESPIC_OK) {
            std::cerr << "Output::fields: snapshot " << J.ticket << " lost" << std::endl;
            return;
        }
        write_fields(J, snap);
    });
}

void Output::screenOutput(World &world, std::vector<Species> &species) {
    std::cout << "ts: " << world.getTs();
    for (Species &sp : species) std::cout << std::setprecision(3) << "\t " << sp.name << ":" << sp.getNp();
    std::cout << std::endl;
}

/* Output::particles, ch4/Output.cpp:175-228: every particle past a running
 * counter of num_parts / np, from the host mirror of the species */
void Output::particles(World &world, std::vector<Species> &species, int num_parts) {
    for (Species &sp : species) {
        std::stringstream name;
        name << "results/parts_" << sp.name << "_" << std::setfill('0') << std::setw(5) << world.getTs() << ".vtp";
        std::ofstream out(name.str());
        if (!out.is_open()) {
            std::cerr << "Could not open " << name.str() << std::endl;
            return;
        }
        double dp = num_parts / (double)sp.getNp();
        double counter = 0;
        std::vector<Particle *> to_output;
        for (Particle &part : sp.particles) {
            counter += dp;
            if (counter > 1) {
                to_output.emplace_back(&part);
                counter = -1;
            }
        }
        out << "<?xml version=\"1.0\"?>\n";
        out << "<VTKFile type=\"PolyData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
        out << "<PolyData>\n";
        out << "<Piece NumberOfPoints=\"" << to_output.size() << "\" NumberOfVerts=\"0\" NumberOfLines=\"0\" ";
        out << "NumberOfStrips=\"0\" NumberOfCells=\"0\">\n";
        out << "<Points>\n";
        out << "<DataArray type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (Particle *part : to_output) out << part->pos << "\n";
        out << "</DataArray>\n";
        out << "</Points>\n";
        out << "<PointData>\n";
        out << "<DataArray Name=\"vel." << sp.name << "\" type=\"Float64\" NumberOfComponents=\"3\" format=\"ascii\">\n";
        for (Particle *part : to_output) out << part->vel << "\n";
        out << "</DataArray>\n";
        out << "</PointData>\n";
        out << "</Piece>\n";
        out << "</PolyData>\n";
        out << "</VTKFile>\n";
        out.close();
    }
}

/* Output::diagOutput, ch3/ver2/Output.cpp:96-132: runtime_diags.csv */
void Output::diagOutput(World &world, std::vector<Species> &species) {
    if (!f_diag.is_open()) {
        f_diag.open("runtime_diags.csv");
        f_diag << "ts,time,wall_time";
        for (Species &sp : species)
            f_diag << ",mp_count." << sp.name << ",real_count." << sp.name << ",px." << sp.name << ",py." << sp.name
                   << ",pz." << sp.name << ",KE." << sp.name;
        f_diag << ",PE,E_total" << std::endl;
    }
    f_diag << world.getTs() << "," << world.getTime() << "," << world.getWallTime();
    double tot_KE = 0;
    for (Species &sp : species) {
        double KE = sp.getKE();
        tot_KE += KE;
        double3 mom = sp.getMomentum();
        f_diag << "," << sp.getNp() << "," << sp.getRealCount() << "," << mom[0] << "," << mom[1] << "," << mom[2]
               << "," << KE;
    }
    double PE = world.getPE();
    f_diag << "," << PE << "," << (tot_KE + PE) << "\n";
    if (world.getTs() % 25 == 0) f_diag.flush();
}
