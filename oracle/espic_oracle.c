/*
 * espic_oracle.c -- CPU restatement of the ES-PIC hot path of "Plasma
 * Simulations by Example".  TEST INFRASTRUCTURE ONLY: the parity checker for
 * the CUDA path, never part of the product.  See espic_oracle.h for the data
 * conventions.  Each function cites the reference code it restates.
 *
 * Deliberate, documented departures from the reference (the CUDA path makes
 * the same ones, so the two agree):
 *  - gather/scatter clamp the cell index to [0, n-2] per axis.  The reference
 *    reads and writes index n when a particle sits exactly on the max face
 *    after a one-bounce reflection (ch2/Species.cpp:32-36 with
 *    ch2/Field.h:164-208); the clamp keeps the same interpolation weights
 *    (di = 1) without the out-of-bounds access.
 *  - node volumes are allocated (ni,nj,nk); the reference allocates
 *    (ni,nk,nk) (ch2/World.cpp:16) which is only safe when nj <= nk.
 */
#include "espic_oracle.h"
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define NODE(g, i, j, k) ((int64_t)(k) * (g)->ni * (g)->nj + (int64_t)(j) * (g)->ni + (i))

/* ------------------------------------------------------------------------ */
/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as
 * easy as 1, 2, 3", SC'11).  Counter = (index/2 lo, hi, stream lo, hi),
 * key = seed.  Each block gives two 53-bit uniforms in [0,1).             */
void eo_philox4x32(uint32_t c[4], const uint32_t key[2]) {
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c[0];
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c[1] ^ k0;
        uint32_t n2 = hi0 ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = lo1;
        c[2] = n2;
        c[3] = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

static double u53(uint32_t a, uint32_t b) {
    uint64_t x = (((uint64_t)a << 32) | b) >> 11;
    return (double)x * (1.0 / 9007199254740992.0);
}

double eo_philox_uniform(uint64_t seed, uint64_t stream, uint64_t index) {
    uint64_t blk = index >> 1;
    uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)stream,
                     (uint32_t)(stream >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    eo_philox4x32(c, key);
    return (index & 1) ? u53(c[2], c[3]) : u53(c[0], c[1]);
}

void eo_philox_uniforms(uint64_t seed, uint64_t stream, uint64_t first, int64_t n, double *out) {
    for (int64_t i = 0; i < n; i++) out[i] = eo_philox_uniform(seed, stream, first + (uint64_t)i);
}

/* ------------------------------------------------------------------------ */
/* World::setExtents, ch2/World.cpp:22-36 */
void eo_grid_set(eo_grid *g, int ni, int nj, int nk, const double x0[3], const double xm[3]) {
    int nn[3] = {ni, nj, nk};
    g->ni = ni;
    g->nj = nj;
    g->nk = nk;
    g->pad = 0;
    for (int d = 0; d < 3; d++) {
        g->x0[d] = x0[d];
        g->xm[d] = xm[d];
        g->dh[d] = (xm[d] - x0[d]) / (nn[d] - 1);
    }
}

/* World::computeNodeVolumes, ch2/World.cpp:58-69 */
void eo_node_volumes(const eo_grid *g, double *vol) {
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++)
            for (int k = 0; k < g->nk; k++) {
                double V = g->dh[0] * g->dh[1] * g->dh[2];
                if (i == 0 || i == g->ni - 1) V *= 0.5;
                if (j == 0 || j == g->nj - 1) V *= 0.5;
                if (k == 0 || k == g->nk - 1) V *= 0.5;
                vol[NODE(g, i, j, k)] = V;
            }
}

/* World::XtoL, ch2/World.h:72-78 */
void eo_xtol(const eo_grid *g, const double x[3], double lc[3]) {
    for (int d = 0; d < 3; d++) lc[d] = (x[d] - g->x0[d]) / g->dh[d];
}

/* World::inBounds, ch2/World.h:59-63 */
int eo_in_bounds(const eo_grid *g, const double x[3]) {
    for (int d = 0; d < 3; d++)
        if (x[d] < g->x0[d] || x[d] >= g->xm[d]) return 0;
    return 1;
}

static inline int clampi(int i, int n) {
    if (i < 0) i = 0;
    if (i > n - 2) i = n - 2;
    return i;
}

/* Cell index and in-cell fraction: (int) truncation as in Field_::gather,
 * ch2/Field.h:188-196, plus the index clamp described at the top. */
static inline void cell_of(const eo_grid *g, const double lc[3], int ijk[3], double f[3]) {
    int n[3] = {g->ni, g->nj, g->nk};
    for (int d = 0; d < 3; d++) {
        int i = clampi((int)lc[d], n[d]);
        ijk[d] = i;
        f[d] = lc[d] - i;
    }
}

/* Field_<double3>::gather, ch2/Field.h:186-208: 8 terms in the reference's
 * corner order, each term ((E*(1-di))*(1-dj))*(1-dk), summed left to right. */
void eo_gather3(const eo_grid *g, const double *ef, const double lc[3], double out[3]) {
    int c[3];
    double f[3];
    cell_of(g, lc, c, f);
    double di = f[0], dj = f[1], dk = f[2];
    int64_t n000 = NODE(g, c[0], c[1], c[2]);
    int64_t sx = 1, sy = g->ni, sz = (int64_t)g->ni * g->nj;
    int64_t idx[8] = {n000,           n000 + sx,           n000 + sx + sy,      n000 + sy,
                      n000 + sz,      n000 + sx + sz,      n000 + sx + sy + sz, n000 + sy + sz};
    for (int d = 0; d < 3; d++) {
        double v = ef[idx[0] * 3 + d] * (1 - di) * (1 - dj) * (1 - dk) +
                   ef[idx[1] * 3 + d] * (di) * (1 - dj) * (1 - dk) +
                   ef[idx[2] * 3 + d] * (di) * (dj) * (1 - dk) +
                   ef[idx[3] * 3 + d] * (1 - di) * (dj) * (1 - dk) +
                   ef[idx[4] * 3 + d] * (1 - di) * (1 - dj) * (dk) +
                   ef[idx[5] * 3 + d] * (di) * (1 - dj) * (dk) +
                   ef[idx[6] * 3 + d] * (di) * (dj) * (dk) +
                   ef[idx[7] * 3 + d] * (1 - di) * (dj) * (dk);
        out[d] = v;
    }
}

/* ------------------------------------------------------------------------ */
/* Species::advance (box), ch2/Species.cpp:7-38: gather, v += E*(dt*q/m),
 * x += v*dt, one-bounce mirror reflection on every wall. */
void eo_push_box(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                 double *P, int64_t stride, int64_t n) {
    double s = dt * charge / mass;
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        double lc[3], e[3];
        eo_xtol(g, x, lc);
        eo_gather3(g, ef, lc, e);
        for (int d = 0; d < 3; d++) v[d] += e[d] * s;
        for (int d = 0; d < 3; d++) x[d] += v[d] * dt;
        for (int d = 0; d < 3; d++) {
            if (x[d] < g->x0[d]) {
                x[d] = 2 * g->x0[d] - x[d];
                v[d] *= -1.0;
            } else if (x[d] >= g->xm[d]) {
                x[d] = 2 * g->xm[d] - x[d];
                v[d] *= -1.0;
            }
        }
        for (int d = 0; d < 3; d++) {
            P[d * stride + p] = x[d];
            P[(3 + d) * stride + p] = v[d];
        }
    }
}

/* World::inSphere, ch3/ver2/World.cpp:119-126.  sphere = {cx, cy, cz, r^2}. */
static inline int in_sphere(const double sphere[4], const double x[3]) {
    double r0 = x[0] - sphere[0], r1 = x[1] - sphere[1], r2 = x[2] - sphere[2];
    double rm2 = r0 * r0 + r1 * r1 + r2 * r2;
    return rm2 <= sphere[3];
}

/* Species::advance (sphere), ch3/ver2/Species.cpp:7-33: same push; a particle
 * inside the sphere or out of the domain gets mpw = 0.  Returns the number
 * killed.  Compaction is a separate call. */
int64_t eo_push_sphere(const eo_grid *g, const double *ef, const double sphere[4], double charge,
                       double mass, double dt, double *P, int64_t stride, int64_t n) {
    double s = dt * charge / mass;
    int64_t killed = 0;
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        double lc[3], e[3];
        eo_xtol(g, x, lc);
        eo_gather3(g, ef, lc, e);
        for (int d = 0; d < 3; d++) v[d] += e[d] * s;
        for (int d = 0; d < 3; d++) x[d] += v[d] * dt;
        for (int d = 0; d < 3; d++) {
            P[d * stride + p] = x[d];
            P[(3 + d) * stride + p] = v[d];
        }
        if (in_sphere(sphere, x) || !eo_in_bounds(g, x)) {
            P[6 * stride + p] = 0;
            killed++;
        }
    }
    return killed;
}

static inline void copy_particle(double *P, int64_t stride, int64_t dst, int64_t src) {
    for (int c = 0; c < 7; c++) P[c * stride + dst] = P[c * stride + src];
}

/* Removal step of ch3/ver2/Species.cpp:35-46: a dead slot (mpw <= 0) is
 * filled with the last particle and re-checked. */
int64_t eo_compact_swap_last(double *P, int64_t stride, int64_t n) {
    int64_t np = n;
    for (int64_t p = 0; p < np; p++) {
        if (P[6 * stride + p] > 0) continue;
        copy_particle(P, stride, p, np - 1);
        np--;
        p--;
    }
    return np;
}

/* The CUDA path's deterministic in-place compaction: with n_new live
 * particles, the r-th dead slot below n_new (in index order) receives the
 * r-th live particle at or above n_new.  Same survivors as the reference,
 * different order. */
int64_t eo_compact_holes(double *P, int64_t stride, int64_t n) {
    int64_t alive = 0;
    for (int64_t p = 0; p < n; p++) alive += P[6 * stride + p] > 0;
    int64_t hole = 0;
    for (int64_t src = alive; src < n; src++) {
        if (!(P[6 * stride + src] > 0)) continue;
        while (P[6 * stride + hole] > 0) hole++;
        copy_particle(P, stride, hole, src);
        hole++;
    }
    return alive;
}

/* Species::addParticle, ch2/Species.cpp:55-71: reject outside [x0,xm),
 * rewind v by (q/m)*E*(dt/2), append. */
int64_t eo_add_particles(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                         const double *pos3, const double *vel3, const double *w, int64_t n,
                         double *P, int64_t stride, int64_t np0, int64_t cap) {
    int64_t np = np0;
    double qm = charge / mass;
    for (int64_t p = 0; p < n; p++) {
        const double *x = pos3 + 3 * p;
        if (!eo_in_bounds(g, x)) continue;
        if (np >= cap) return -1;
        double lc[3], e[3], v[3];
        eo_xtol(g, x, lc);
        eo_gather3(g, ef, lc, e);
        for (int d = 0; d < 3; d++) v[d] = vel3[3 * p + d] - e[d] * qm * (0.5 * dt);
        for (int d = 0; d < 3; d++) {
            P[d * stride + np] = x[d];
            P[(3 + d) * stride + np] = v[d];
        }
        P[6 * stride + np] = w[p];
        np++;
    }
    return np;
}

/* Species::loadParticlesBox, ch2/Species.cpp:74-97, with the uniforms given
 * explicitly (3 per particle, x then y then z). */
int64_t eo_load_box(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                    const double x1[3], const double x2[3], double num_den, int64_t num_mp,
                    const double *u, double *P, int64_t stride, int64_t np0, int64_t cap) {
    double box_vol = (x2[0] - x1[0]) * (x2[1] - x1[1]) * (x2[2] - x1[2]);
    double num_real = num_den * box_vol;
    double mpw = num_real / (double)num_mp;
    int64_t np = np0;
    for (int64_t p = 0; p < num_mp; p++) {
        double pos[3], vel[3] = {0, 0, 0};
        for (int d = 0; d < 3; d++) pos[d] = x1[d] + u[3 * p + d] * (x2[d] - x1[d]);
        np = eo_add_particles(g, ef, charge, mass, dt, pos, vel, &mpw, 1, P, stride, np, cap);
        if (np < 0) return -1;
    }
    return np;
}

/* Species::loadParticlesBoxQS, ch2/Species.cpp:101-141 */
int64_t eo_load_box_qs(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       const double x1[3], const double x2[3], double num_den, const int num_mp[3],
                       double *P, int64_t stride, int64_t np0, int64_t cap) {
    double box_vol = (x2[0] - x1[0]) * (x2[1] - x1[1]) * (x2[2] - x1[2]);
    int num_mp_tot = (num_mp[0] - 1) * (num_mp[1] - 1) * (num_mp[2] - 1);
    double num_real = num_den * box_vol;
    double mpw = num_real / num_mp_tot;
    double di = (x2[0] - x1[0]) / (num_mp[0] - 1);
    double dj = (x2[1] - x1[1]) / (num_mp[1] - 1);
    double dk = (x2[2] - x1[2]) / (num_mp[2] - 1);
    int64_t np = np0;
    for (int i = 0; i < num_mp[0]; i++)
        for (int j = 0; j < num_mp[1]; j++)
            for (int k = 0; k < num_mp[2]; k++) {
                double pos[3], vel[3] = {0, 0, 0};
                pos[0] = x1[0] + i * di;
                pos[1] = x1[1] + j * dj;
                pos[2] = x1[2] + k * dk;
                if (pos[0] == x2[0]) pos[0] -= 1e-4 * di;
                if (pos[1] == x2[1]) pos[1] -= 1e-4 * dj;
                if (pos[2] == x2[2]) pos[2] -= 1e-4 * dk;
                double w = 1;
                if (i == 0 || i == num_mp[0] - 1) w *= 0.5;
                if (j == 0 || j == num_mp[1] - 1) w *= 0.5;
                if (k == 0 || k == num_mp[2] - 1) w *= 0.5;
                double ww = mpw * w;
                np = eo_add_particles(g, ef, charge, mass, dt, pos, vel, &ww, 1, P, stride, np, cap);
                if (np < 0) return -1;
            }
    return np;
}

/* The CUDA path's thermal box loader (an extension with no reference
 * counterpart): positions as loadParticlesBox, velocities vd + sigma * N(0,1)
 * by Box-Muller with sigma = sqrt(K T / m); 7 uniforms per particle. */
int64_t eo_load_box_thermal(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                            const double x1[3], const double x2[3], double mpw, int64_t num_mp,
                            const double vd[3], double temp, const double *u, double *P, int64_t stride,
                            int64_t np0, int64_t cap) {
    double sigma = sqrt(EO_K * temp / mass);
    int64_t np = np0;
    for (int64_t p = 0; p < num_mp; p++) {
        const double *up = u + 7 * p;
        double pos[3], vel[3];
        for (int d = 0; d < 3; d++) pos[d] = x1[d] + up[d] * (x2[d] - x1[d]);
        double r1 = sqrt(-2.0 * log(1.0 - up[3])), a1 = 2 * EO_PI * up[4];
        double r2 = sqrt(-2.0 * log(1.0 - up[5])), a2 = 2 * EO_PI * up[6];
        vel[0] = vd[0] + sigma * (r1 * cos(a1));
        vel[1] = vd[1] + sigma * (r1 * sin(a1));
        vel[2] = vd[2] + sigma * (r2 * cos(a2));
        np = eo_add_particles(g, ef, charge, mass, dt, pos, vel, &mpw, 1, P, stride, np, cap);
        if (np < 0) return -1;
    }
    return np;
}

/* Number of macroparticles a beam source creates this step,
 * ch3/ver2/Source.cpp:7-18: (int)(n*v*A*dt/mpw0 + U). */
int eo_inject_count(const eo_grid *g, double dt, double mpw0, double v_drift, double den,
                    double u0) {
    double Lx = g->dh[0] * (g->ni - 1);
    double Ly = g->dh[1] * (g->nj - 1);
    double A = Lx * Ly;
    double num_real = den * v_drift * A * dt;
    return (int)(num_real / mpw0 + u0);
}

/* ColdBeamSource::sample, ch3/ver2/Source.cpp:4-27.  Uniform order: count,
 * then (x, y) per particle. */
int64_t eo_inject_cold(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       double mpw0, double v_drift, double den, const double *u, int64_t *u_used,
                       double *P, int64_t stride, int64_t np0, int64_t cap) {
    double Lx = g->dh[0] * (g->ni - 1);
    double Ly = g->dh[1] * (g->nj - 1);
    int num_sim = eo_inject_count(g, dt, mpw0, v_drift, den, u[0]);
    int64_t np = np0;
    for (int i = 0; i < num_sim; i++) {
        double pos[3] = {g->x0[0] + u[1 + 2 * i] * Lx, g->x0[1] + u[2 + 2 * i] * Ly, g->x0[2]};
        double vel[3] = {0, 0, v_drift};
        np = eo_add_particles(g, ef, charge, mass, dt, pos, vel, &mpw0, 1, P, stride, np, cap);
        if (np < 0) return -1;
    }
    if (u_used) *u_used = 1 + 2 * (int64_t)num_sim;
    return np;
}

/* Species::sampleVth and Species::sampleIsotropicVel, ch4/Species.cpp:149-175.
 * u: theta, r, then 9 uniforms for the three speed components. */
static void isotropic_vel(double mass, double temp, const double *u, double out[3]) {
    double theta = 2 * EO_PI * u[0];
    double r = -1.0 + 2 * u[1];
    double a = sqrt(1 - r * r);
    double d[3] = {r, cos(theta) * a, sin(theta) * a};
    double v_th = sqrt(2 * EO_K * temp / mass);
    double v1 = v_th * (u[2] + u[3] + u[4] - 1.5);
    double v2 = v_th * (u[5] + u[6] + u[7] - 1.5);
    double v3 = v_th * (u[8] + u[9] + u[10] - 1.5);
    double speed = 3 / sqrt(2 + 2 + 2) * sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    for (int c = 0; c < 3; c++) out[c] = d[c] * speed;
}

/* WarmBeamSource::sample, ch4/Source.cpp:31-55: cold-beam positions plus an
 * isotropic thermal velocity, drift added to z.  13 uniforms per particle. */
int64_t eo_inject_warm(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       double mpw0, double v_drift, double den, double temp, const double *u,
                       int64_t *u_used, double *P, int64_t stride, int64_t np0, int64_t cap) {
    double Lx = g->dh[0] * (g->ni - 1);
    double Ly = g->dh[1] * (g->nj - 1);
    int num_sim = eo_inject_count(g, dt, mpw0, v_drift, den, u[0]);
    int64_t np = np0;
    for (int i = 0; i < num_sim; i++) {
        const double *ui = u + 1 + 13 * (int64_t)i;
        double pos[3] = {g->x0[0] + ui[0] * Lx, g->x0[1] + ui[1] * Ly, g->x0[2]};
        double vel[3];
        isotropic_vel(mass, temp, ui + 2, vel);
        vel[2] += v_drift;
        np = eo_add_particles(g, ef, charge, mass, dt, pos, vel, &mpw0, 1, P, stride, np, cap);
        if (np < 0) return -1;
    }
    if (u_used) *u_used = 1 + 13 * (int64_t)num_sim;
    return np;
}

/* Source::sample of ch9/MPI (ch9/MPI/src/Source.cpp:5-72) and a
 * drifting-Maxwellian beam.  mode 2: isotropic direction (theta, R) at the
 * speed sqrt(2 Kb T / m) with ch9/MPI's Kb = 1.3806488e-23 and PI = acos(-1),
 * drift added to z, v_z < 0 reflected; 4 uniforms per particle (x, y, theta,
 * R).  mode 3: normal components of deviation sqrt(k T / m) by Box-Muller
 * (radius sqrt(-2 ln(1 - u)), angle 2 pi u), drift added, v_z < 0 reflected;
 * 6 uniforms per particle.  The count is the remainder count of ch9/MPI
 * (*rem carried) when rem != NULL, else (int)(N + u[0]).  The rewind is that
 * of addParticle here and of ch9/MPI/src/Source.cpp:61-68 (same expression). */
/* World::XtoC, ch4/World.h:79-98: truncated logical coordinates */
static int64_t dsmc_cell(const eo_grid *g, const double x[3]) {
    int ijk[3];
    for (int d = 0; d < 3; d++) ijk[d] = (int)((x[d] - g->x0[d]) / g->dh[d]);
    return (int64_t)ijk[2] * (g->nj - 1) * (g->ni - 1) + (int64_t)ijk[1] * (g->ni - 1) + ijk[0];
}

/* vec3 magnitude, ch4/Field.h:21-26: sqrt of ((0 + x x) + y y) + z z */
static double dsmc_mag(const double v[3]) {
    double s = 0;
    for (int i = 0; i < 3; i++) s += v[i] * v[i];
    return sqrt(s);
}

/* DSMC_MEX::collide, ch4/Collisions.cpp:84-105 (isotropic scattering) */
static void dsmc_collide(double *v1, double *v2, double m1, double m2, double u_chi, double u_eps) {
    double cm[3], cr[3];
    for (int i = 0; i < 3; i++) cm[i] = (v1[i] * m1 + v2[i] * m2) / (m1 + m2);
    for (int i = 0; i < 3; i++) cr[i] = v1[i] - v2[i];
    const double cr_mag = dsmc_mag(cr);
    const double cos_chi = 2 * u_chi - 1;
    const double sin_chi = sqrt(1 - cos_chi * cos_chi);
    const double eps = 2 * EO_PI * u_eps;
    cr[0] = cr_mag * cos_chi;
    cr[1] = cr_mag * sin_chi * cos(eps);
    cr[2] = cr_mag * sin_chi * sin(eps);
    const double s1 = m2 / (m1 + m2), s2 = m1 / (m1 + m2);
    for (int i = 0; i < 3; i++) {
        v1[i] = cm[i] + cr[i] * s1;
        v2[i] = cm[i] - cr[i] * s2;
    }
}

int64_t eo_dsmc_mex(const eo_grid *g, double mass, double mpw0, double dt, const double c[4],
                    double *sigma_cr_max, double *P, int64_t stride, int64_t n, const double *u, int64_t nu,
                    int64_t *u_used, int64_t *cell_off) {
    const int64_t n_cells = (int64_t)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    int64_t *start = (int64_t *)calloc((size_t)n_cells + 1, sizeof(int64_t));
    int64_t *fill = (int64_t *)calloc((size_t)n_cells + 1, sizeof(int64_t));
    int64_t *cellof = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    int64_t *list = (int64_t *)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    /* the particles of each cell in particle order (parts_in_cell) */
    for (int64_t p = 0; p < n; p++) {
        const double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        cellof[p] = dsmc_cell(g, x);
        start[cellof[p] + 1]++;
    }
    for (int64_t cc = 0; cc < n_cells; cc++) start[cc + 1] += start[cc];
    for (int64_t p = 0; p < n; p++) list[start[cellof[p]] + fill[cellof[p]]++] = p;
    double sigma_cr_max_temp = 0;
    const double dV = g->dh[0] * g->dh[1] * g->dh[2];
    const double Fn = mpw0;
    int64_t num_cols = 0, k = 0;
#define DSMC_U() (k < nu ? u[k++] : (k++, -1.0))
    for (int64_t cc = 0; cc < n_cells; cc++) {
        if (cell_off) cell_off[cc] = k;
        const int64_t *parts = list + start[cc];
        const int np = (int)(start[cc + 1] - start[cc]);
        if (np < 2) continue;
        const double ng_f = 0.5 * np * np * Fn * (*sigma_cr_max) * dt / dV;
        const int ng = (int)(ng_f + 0.5);
        for (int gg = 0; gg < ng; gg++) {
            const int p1 = (int)(DSMC_U() * np);
            int p2;
            do {
                p2 = (int)(DSMC_U() * np);
            } while (p2 == p1 && k <= nu);
            const int64_t a = parts[p1], b = parts[p2];
            double cr_vec[3];
            for (int d = 0; d < 3; d++) cr_vec[d] = P[(3 + d) * stride + a] - P[(3 + d) * stride + b];
            const double cr = dsmc_mag(cr_vec);
            /* DSMC_MEX::evalSigma, ch4/Collisions.h:64-67 */
            const double sigma = EO_PI * c[0] * c[0] * pow(c[2] / (cr * cr), c[1] - 0.5) / c[3];
            const double sigma_cr = sigma * cr;
            if (sigma_cr > sigma_cr_max_temp) sigma_cr_max_temp = sigma_cr;
            const double Pc = sigma_cr / (*sigma_cr_max);
            if (Pc > DSMC_U()) {
                num_cols++;
                double v1[3], v2[3];
                for (int d = 0; d < 3; d++) {
                    v1[d] = P[(3 + d) * stride + a];
                    v2[d] = P[(3 + d) * stride + b];
                }
                const double u_chi = DSMC_U(), u_eps = DSMC_U();
                dsmc_collide(v1, v2, mass, mass, u_chi, u_eps);
                for (int d = 0; d < 3; d++) {
                    P[(3 + d) * stride + a] = v1[d];
                    P[(3 + d) * stride + b] = v2[d];
                }
            }
        }
    }
#undef DSMC_U
    if (cell_off) cell_off[n_cells] = k;
    if (num_cols) *sigma_cr_max = sigma_cr_max_temp;
    free(start);
    free(fill);
    free(cellof);
    free(list);
    if (u_used) *u_used = k;
    return k > nu ? -1 : num_cols;
}

int64_t eo_inject_beam(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       double mpw0, double v_drift, double den, double temp, int mode, double *rem,
                       const double *u, int64_t *u_used, double *P, int64_t stride, int64_t np0, int64_t cap) {
    const double pi = acos(-1.0);
    double Lx = g->dh[0] * (g->ni - 1);
    double Ly = g->dh[1] * (g->nj - 1);
    int num_sim;
    if (rem) {
        /* the remainder count of ch9/MPI/src/Source.cpp:10-27, in its order */
        double area = (g->ni - 1) * g->dh[0] * (g->nj - 1) * g->dh[1];
        double num_per_sec = den * v_drift * area;
        double num_real = num_per_sec * dt;
        double f = num_real / mpw0 + *rem;
        num_sim = (int)f;
        *rem = f - num_sim;
    } else {
        num_sim = eo_inject_count(g, dt, mpw0, v_drift, den, u[0]);
    }
    const int upp = mode == 2 ? 4 : 6;
    int64_t np = np0;
    for (int i = 0; i < num_sim; i++) {
        const double *ui = u + 1 + upp * (int64_t)i;
        double pos[3] = {g->x0[0] + ui[0] * Lx, g->x0[1] + ui[1] * Ly, g->x0[2]};
        if (mode == 2) { /* x0 + U (ni-1) dh, ch9/MPI/src/Source.cpp:33-35 */
            pos[0] = g->x0[0] + ui[0] * (g->ni - 1) * g->dh[0];
            pos[1] = g->x0[1] + ui[1] * (g->nj - 1) * g->dh[1];
        }
        double vel[3];
        if (mode == 2) {
            double v_th = sqrt(2 * 1.3806488e-23 * temp / mass);
            double theta = 2 * pi * ui[2];
            double R = -1.0 + 2 * ui[3];
            double a = sqrt(1 - R * R);
            vel[0] = v_th * (cos(theta) * a);
            vel[1] = v_th * (sin(theta) * a);
            vel[2] = v_th * R + v_drift;
        } else {
            double sig = sqrt(EO_K * temp / mass);
            double r1 = sqrt(-2.0 * log(1.0 - ui[2])), a1 = 2 * pi * ui[3];
            double r2 = sqrt(-2.0 * log(1.0 - ui[4])), a2 = 2 * pi * ui[5];
            vel[0] = sig * (r1 * cos(a1));
            vel[1] = sig * (r1 * sin(a1));
            vel[2] = sig * (r2 * cos(a2)) + v_drift;
        }
        if (vel[2] < 0) vel[2] = -vel[2];
        np = eo_add_particles(g, ef, charge, mass, dt, pos, vel, &mpw0, 1, P, stride, np, cap);
        if (np < 0) return -1;
    }
    if (u_used) *u_used = 1 + upp * (int64_t)num_sim;
    return np;
}

/* ------------------------------------------------------------------------ */
/* Corner weights of Field_::scatter, ch2/Field.h:164-183, in the reference's
 * corner order: value*(1-di)*(1-dj)*(1-dk) evaluated left to right. */
static inline void cic_weights(double value, double di, double dj, double dk, double w[8]) {
    w[0] = value * (1 - di) * (1 - dj) * (1 - dk);
    w[1] = value * (di) * (1 - dj) * (1 - dk);
    w[2] = value * (di) * (dj) * (1 - dk);
    w[3] = value * (1 - di) * (dj) * (1 - dk);
    w[4] = value * (1 - di) * (1 - dj) * (dk);
    w[5] = value * (di) * (1 - dj) * (dk);
    w[6] = value * (di) * (dj) * (dk);
    w[7] = value * (1 - di) * (dj) * (dk);
}

static inline void cic_nodes(const eo_grid *g, const int c[3], int64_t idx[8]) {
    int64_t n000 = NODE(g, c[0], c[1], c[2]);
    int64_t sx = 1, sy = g->ni, sz = (int64_t)g->ni * g->nj;
    idx[0] = n000;
    idx[1] = n000 + sx;
    idx[2] = n000 + sx + sy;
    idx[3] = n000 + sy;
    idx[4] = n000 + sz;
    idx[5] = n000 + sx + sz;
    idx[6] = n000 + sx + sy + sz;
    idx[7] = n000 + sy + sz;
}

/* Species::computeNumberDensity scatter loop, ch2/Species.cpp:41-49, FP64 sum
 * in particle order (the reference's own arithmetic). */
void eo_deposit_fp64(const eo_grid *g, const double *P, int64_t stride, int64_t n, double *acc) {
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double lc[3], f[3], w[8];
        int c[3];
        int64_t idx[8];
        eo_xtol(g, x, lc);
        cell_of(g, lc, c, f);
        cic_weights(P[6 * stride + p], f[0], f[1], f[2], w);
        cic_nodes(g, c, idx);
        for (int m = 0; m < 8; m++) acc[idx[m]] += w[m];
    }
}

/* The CUDA path's deposit: each corner weight is rounded once to a 64-bit
 * integer in units of 1/fx (fx a power of two) and summed exactly, so the
 * total does not depend on particle order. */
void eo_deposit_fixed(const eo_grid *g, const double *P, int64_t stride, int64_t n, double fx,
                      int64_t *acc) {
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double lc[3], f[3], w[8];
        int c[3];
        int64_t idx[8];
        eo_xtol(g, x, lc);
        cell_of(g, lc, c, f);
        cic_weights(P[6 * stride + p], f[0], f[1], f[2], w);
        cic_nodes(g, c, idx);
        for (int m = 0; m < 8; m++) acc[idx[m]] += (int64_t)llrint(w[m] * fx);
    }
}

/* Field_::operator/=, ch2/Field.h:125-134: divide, or 0 where vol == 0. */
void eo_divide_volume(int64_t nn, double *den, const double *vol) {
    for (int64_t u = 0; u < nn; u++) {
        if (vol[u] != 0)
            den[u] /= vol[u];
        else
            den[u] = 0;
    }
}

void eo_density_from_fixed(int64_t nn, const int64_t *acc, double inv_fx, const double *vol,
                           double *den) {
    for (int64_t u = 0; u < nn; u++) den[u] = (double)acc[u] * inv_fx;
    eo_divide_volume(nn, den, vol);
}

/* World::computeChargeDensity, ch2/World.cpp:46-54: rho = 0; rho += q_s*den_s
 * for each charged species.  dens is [ns][nn]. */
void eo_charge_density(int64_t nn, int ns, const double *charges, const double *dens, double *rho) {
    for (int64_t u = 0; u < nn; u++) rho[u] = 0;
    for (int s = 0; s < ns; s++) {
        if (charges[s] == 0) continue;
        const double *d = dens + (int64_t)s * nn;
        for (int64_t u = 0; u < nn; u++) rho[u] += d[u] * charges[s];
    }
}

/* Exponent S of the fixed-point scale fx = 2^S: the largest S with
 * capacity * weight_bound * 2^S <= 2^62, so that no node total can overflow
 * a signed 64-bit integer; capped at 52. */
int eo_fixed_scale_exponent(double weight_bound, int64_t capacity) {
    if (capacity < 1) capacity = 1;
    if (!(weight_bound > 0)) weight_bound = 1;
    double lim = ldexp(1.0, 62) / ((double)capacity * weight_bound);
    int e;
    frexp(lim, &e); /* lim = m*2^e, m in [0.5,1) -> 2^(e-1) <= lim */
    int S = e - 1;
    if (S > 52) S = 52;
    return S;
}

/* ------------------------------------------------------------------------ */
/* Residual of PotentialSolver::solve, ch2/PotentialSolver.cpp:44-61. */
double eo_residual_box(const eo_grid *g, const double *phi, const double *rho) {
    double idx2 = 1.0 / (g->dh[0] * g->dh[0]);
    double idy2 = 1.0 / (g->dh[1] * g->dh[1]);
    double idz2 = 1.0 / (g->dh[2] * g->dh[2]);
    int64_t sy = g->ni, sz = (int64_t)g->ni * g->nj;
    double sum = 0;
    for (int i = 1; i < g->ni - 1; i++)
        for (int j = 1; j < g->nj - 1; j++)
            for (int k = 1; k < g->nk - 1; k++) {
                int64_t u = NODE(g, i, j, k);
                double R = -phi[u] * (2 * idx2 + 2 * idy2 + 2 * idz2) + rho[u] / EO_EPS_0 +
                           idx2 * (phi[u - 1] + phi[u + 1]) + idy2 * (phi[u - sy] + phi[u + sy]) +
                           idz2 * (phi[u - sz] + phi[u + sz]);
                sum += R * R;
            }
    return sqrt(sum / (g->ni * g->nj * g->nk));
}

static inline void sor_box_node(const eo_grid *g, double *phi, const double *rho, int64_t u,
                                double idx2, double idy2, double idz2) {
    int64_t sy = g->ni, sz = (int64_t)g->ni * g->nj;
    double phi_new = (rho[u] / EO_EPS_0 + idx2 * (phi[u - 1] + phi[u + 1]) +
                      idy2 * (phi[u - sy] + phi[u + sy]) + idz2 * (phi[u - sz] + phi[u + sz])) /
                     (2 * idx2 + 2 * idy2 + 2 * idz2);
    phi[u] = phi[u] + 1.4 * (phi_new - phi[u]);
}

/* PotentialSolver::solve, ch2/PotentialSolver.cpp:11-67: lexicographic
 * SOR (omega 1.4) over interior nodes, residual every 25 iterations. */
int eo_sor_box_lex(const eo_grid *g, double *phi, const double *rho, int max_it, double tol,
                   double *l2_out, int *it_out) {
    double idx2 = 1.0 / (g->dh[0] * g->dh[0]);
    double idy2 = 1.0 / (g->dh[1] * g->dh[1]);
    double idz2 = 1.0 / (g->dh[2] * g->dh[2]);
    double L2 = 0;
    int conv = 0, it;
    for (it = 0; it < max_it; it++) {
        for (int i = 1; i < g->ni - 1; i++)
            for (int j = 1; j < g->nj - 1; j++)
                for (int k = 1; k < g->nk - 1; k++)
                    sor_box_node(g, phi, rho, NODE(g, i, j, k), idx2, idy2, idz2);
        if (it % 25 == 0) {
            L2 = eo_residual_box(g, phi, rho);
            if (L2 < tol) {
                conv = 1;
                break;
            }
        }
    }
    if (l2_out) *l2_out = L2;
    if (it_out) *it_out = conv ? it + 1 : it;
    return conv;
}

/* The CUDA path's red-black ordering of the same SOR: colour (i+j+k)&1, red
 * (0) then black (1), same node formula, same residual schedule. */
int eo_sor_box_rb(const eo_grid *g, double *phi, const double *rho, int max_it, double tol,
                  double *l2_out, int *it_out) {
    double idx2 = 1.0 / (g->dh[0] * g->dh[0]);
    double idy2 = 1.0 / (g->dh[1] * g->dh[1]);
    double idz2 = 1.0 / (g->dh[2] * g->dh[2]);
    double L2 = 0;
    int conv = 0, it;
    for (it = 0; it < max_it; it++) {
        for (int colour = 0; colour < 2; colour++)
            for (int k = 1; k < g->nk - 1; k++)
                for (int j = 1; j < g->nj - 1; j++)
                    for (int i = 1; i < g->ni - 1; i++)
                        if (((i + j + k) & 1) == colour)
                            sor_box_node(g, phi, rho, NODE(g, i, j, k), idx2, idy2, idz2);
        if (it % 25 == 0) {
            L2 = eo_residual_box(g, phi, rho);
            if (L2 < tol) {
                conv = 1;
                break;
            }
        }
    }
    if (l2_out) *l2_out = L2;
    if (it_out) *it_out = conv ? it + 1 : it;
    return conv;
}

/* World::addSphere, ch3/ver2/World.cpp:88-106: node position x0 + dh*(i,j,k);
 * nodes inside or on the sphere get object_id 1 and the sphere potential. */
void eo_objects_sphere(const eo_grid *g, const double c[3], double radius, double phi_s, int *obj,
                       double *phi) {
    double sphere[4] = {c[0], c[1], c[2], radius * radius};
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++)
            for (int k = 0; k < g->nk; k++) {
                double l[3] = {(double)i, (double)j, (double)k};
                double x[3];
                for (int d = 0; d < 3; d++) x[d] = g->x0[d] + g->dh[d] * l[d];
                if (in_sphere(sphere, x)) {
                    obj[NODE(g, i, j, k)] = 1;
                    phi[NODE(g, i, j, k)] = phi_s;
                }
            }
}

/* World::addInlet, ch3/ver2/World.cpp:109-116: k = 0 plane is Dirichlet 0 V. */
void eo_objects_inlet(const eo_grid *g, int *obj, double *phi) {
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++) {
            obj[NODE(g, i, j, 0)] = 2;
            phi[NODE(g, i, j, 0)] = 0;
        }
}

/* Immediate Neumann neighbour of a boundary node, in the precedence of
 * PotentialSolver::solveGS, ch3/ver2/PotentialSolver.cpp:359-370; -1 for an
 * interior node. */
static int64_t neumann_next(const eo_grid *g, int i, int j, int k) {
    if (i == 0) return NODE(g, i + 1, j, k);
    if (i == g->ni - 1) return NODE(g, i - 1, j, k);
    if (j == 0) return NODE(g, i, j + 1, k);
    if (j == g->nj - 1) return NODE(g, i, j - 1, k);
    if (k == 0) return NODE(g, i, j, k + 1);
    if (k == g->nk - 1) return NODE(g, i, j, k - 1);
    return -1;
}

/* For each non-Dirichlet boundary node, the end of its chain of Neumann
 * copies (an interior or a Dirichlet node); -1 elsewhere.  At the fixed
 * point of solveGS every boundary node equals its chain end. */
void eo_neumann_targets(const eo_grid *g, const int *obj, int *target) {
    for (int k = 0; k < g->nk; k++)
        for (int j = 0; j < g->nj; j++)
            for (int i = 0; i < g->ni; i++) {
                int64_t u = NODE(g, i, j, k);
                target[u] = -1;
                if (obj[u] > 0) continue;
                int64_t nx = neumann_next(g, i, j, k);
                if (nx < 0) continue;
                int64_t t = nx;
                for (int guard = 0; guard < 8; guard++) {
                    if (obj[t] > 0) break;
                    int ti = (int)(t % g->ni), tj = (int)((t / g->ni) % g->nj),
                        tk = (int)(t / ((int64_t)g->ni * g->nj));
                    int64_t n2 = neumann_next(g, ti, tj, tk);
                    if (n2 < 0) break;
                    t = n2;
                }
                target[u] = (int)t;
            }
}

/* Residual of solveGS, ch3/ver2/PotentialSolver.cpp:394-424. */
double eo_residual_sphere(const eo_grid *g, const double *phi, const double *rho, const int *obj,
                          double phi0, double te0, double n0) {
    double idx2 = 1.0 / (g->dh[0] * g->dh[0]);
    double idy2 = 1.0 / (g->dh[1] * g->dh[1]);
    double idz2 = 1.0 / (g->dh[2] * g->dh[2]);
    int64_t sy = g->ni, sz = (int64_t)g->ni * g->nj;
    double sum = 0;
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++)
            for (int k = 0; k < g->nk; k++) {
                int64_t u = NODE(g, i, j, k);
                if (obj[u] > 0) continue;
                int64_t nb = neumann_next(g, i, j, k);
                double R;
                if (nb >= 0)
                    R = phi[u] - phi[nb];
                else {
                    double ne = n0 * exp((phi[u] - phi0) / te0);
                    R = -phi[u] * (2 * idx2 + 2 * idy2 + 2 * idz2) + (rho[u] - EO_QE * ne) / EO_EPS_0 +
                        idx2 * (phi[u - 1] + phi[u + 1]) + idy2 * (phi[u - sy] + phi[u + sy]) +
                        idz2 * (phi[u - sz] + phi[u + sz]);
                }
                sum += R * R;
            }
    return sqrt(sum / (g->ni * g->nj * g->nk));
}

static inline void gs_sphere_node(const eo_grid *g, double *phi, const double *rho, int64_t u,
                                  double idx2, double idy2, double idz2, double phi0, double te0,
                                  double n0) {
    int64_t sy = g->ni, sz = (int64_t)g->ni * g->nj;
    double ne = n0 * exp((phi[u] - phi0) / te0);
    double phi_new = ((rho[u] - EO_QE * ne) / EO_EPS_0 + idx2 * (phi[u - 1] + phi[u + 1]) +
                      idy2 * (phi[u - sy] + phi[u + sy]) + idz2 * (phi[u - sz] + phi[u + sz])) /
                     (2 * idx2 + 2 * idy2 + 2 * idz2);
    phi[u] = phi[u] + 1.4 * (phi_new - phi[u]);
}

/* PotentialSolver::solveGS, ch3/ver2/PotentialSolver.cpp:334-430:
 * lexicographic nonlinear SOR with Boltzmann electrons. */
int eo_gs_sphere_lex(const eo_grid *g, double *phi, const double *rho, const int *obj, double phi0,
                     double te0, double n0, int max_it, double tol, double *l2_out, int *it_out) {
    double idx2 = 1.0 / (g->dh[0] * g->dh[0]);
    double idy2 = 1.0 / (g->dh[1] * g->dh[1]);
    double idz2 = 1.0 / (g->dh[2] * g->dh[2]);
    double L2 = 0;
    int conv = 0, it;
    for (it = 0; it < max_it; it++) {
        for (int i = 0; i < g->ni; i++)
            for (int j = 0; j < g->nj; j++)
                for (int k = 0; k < g->nk; k++) {
                    int64_t u = NODE(g, i, j, k);
                    if (obj[u] > 0) continue;
                    int64_t nb = neumann_next(g, i, j, k);
                    if (nb >= 0)
                        phi[u] = phi[nb];
                    else
                        gs_sphere_node(g, phi, rho, u, idx2, idy2, idz2, phi0, te0, n0);
                }
        if (it % 25 == 0) {
            L2 = eo_residual_sphere(g, phi, rho, obj, phi0, te0, n0);
            if (L2 < tol) {
                conv = 1;
                break;
            }
        }
    }
    if (l2_out) *l2_out = L2;
    if (it_out) *it_out = conv ? it + 1 : it;
    return conv;
}

/* The CUDA path's red-black form of solveGS: red then black interior
 * non-Dirichlet nodes, then every Neumann node copies its chain end. */
int eo_sor_sphere_rb(const eo_grid *g, double *phi, const double *rho, const int *obj,
                     const int *target, double phi0, double te0, double n0, int max_it, double tol,
                     double *l2_out, int *it_out) {
    double idx2 = 1.0 / (g->dh[0] * g->dh[0]);
    double idy2 = 1.0 / (g->dh[1] * g->dh[1]);
    double idz2 = 1.0 / (g->dh[2] * g->dh[2]);
    int64_t nn = (int64_t)g->ni * g->nj * g->nk;
    double L2 = 0;
    int conv = 0, it;
    for (it = 0; it < max_it; it++) {
        for (int colour = 0; colour < 2; colour++)
            for (int k = 1; k < g->nk - 1; k++)
                for (int j = 1; j < g->nj - 1; j++)
                    for (int i = 1; i < g->ni - 1; i++) {
                        int64_t u = NODE(g, i, j, k);
                        if (((i + j + k) & 1) != colour || obj[u] > 0) continue;
                        gs_sphere_node(g, phi, rho, u, idx2, idy2, idz2, phi0, te0, n0);
                    }
        for (int64_t u = 0; u < nn; u++)
            if (target[u] >= 0) phi[u] = phi[target[u]];
        if (it % 25 == 0) {
            L2 = eo_residual_sphere(g, phi, rho, obj, phi0, te0, n0);
            if (L2 < tol) {
                conv = 1;
                break;
            }
        }
    }
    if (l2_out) *l2_out = L2;
    if (it_out) *it_out = conv ? it + 1 : it;
    return conv;
}

/* PotentialSolver::solveQN, ch3/ver2/PotentialSolver.cpp:204-222 */
void eo_qn(const eo_grid *g, double *phi, const double *rho, const int *obj, double phi0,
           double te0, double n0) {
    double rho0 = n0 * EO_QE;
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++)
            for (int k = 0; k < g->nk; k++) {
                int64_t u = NODE(g, i, j, k);
                if (obj[u] > 0) continue;
                double ratio = rho[u] / rho0;
                if (ratio < 1e-6) ratio = 1e-6;
                phi[u] = phi0 + te0 * log(ratio);
            }
}

/* ---- matrix-free Newton / Jacobi-PCG on the symmetric form of the
 * discrete problem of solveGS (the CUDA path's algorithm).  Unknowns are
 * interior nodes with obj == 0.  L = -Laplacian with Dirichlet neighbours
 * moved to the right-hand side and Neumann neighbours mirrored (a boundary
 * neighbour of an interior node always copies that node), so L is SPD.
 * F(x) = L x - bD + (qe n0/eps0) e^{(x-phi0)/Te} - rho/eps0,
 * J = L + diag((qe n0/(eps0 Te)) e^{(x-phi0)/Te}).  The reference's own
 * Newton-PCG (ch3/ver2/PotentialSolver.cpp:225-331) uses a non-symmetric
 * matrix on which CG breaks down; this form solves the same equations. */
typedef struct {
    const eo_grid *g;
    const int *obj;
    double c[3];
} nk_ctx;

static inline int is_unknown(const nk_ctx *K, int i, int j, int k) {
    const eo_grid *g = K->g;
    if (i < 1 || j < 1 || k < 1 || i > g->ni - 2 || j > g->nj - 2 || k > g->nk - 2) return 0;
    return K->obj[NODE(g, i, j, k)] == 0;
}

/* neighbour kind: 0 unknown, 1 Dirichlet, 2 Neumann boundary */
static inline int nb_kind(const nk_ctx *K, int i, int j, int k) {
    const eo_grid *g = K->g;
    int64_t u = NODE(g, i, j, k);
    if (K->obj[u] > 0) return 1;
    if (i == 0 || j == 0 || k == 0 || i == g->ni - 1 || j == g->nj - 1 || k == g->nk - 1) return 2;
    return 0;
}

static const int NB_OFF[6][3] = {{-1, 0, 0}, {1, 0, 0}, {0, -1, 0}, {0, 1, 0}, {0, 0, -1}, {0, 0, 1}};

/* y = L x on unknowns (x zero elsewhere); diag gets the diagonal of L. */
static void apply_L(const nk_ctx *K, const double *x, double *y, double *diag) {
    const eo_grid *g = K->g;
    for (int k = 1; k < g->nk - 1; k++)
        for (int j = 1; j < g->nj - 1; j++)
            for (int i = 1; i < g->ni - 1; i++) {
                int64_t u = NODE(g, i, j, k);
                if (K->obj[u] != 0) continue;
                double s = 0, d = 0;
                for (int m = 0; m < 6; m++) {
                    int a = i + NB_OFF[m][0], b = j + NB_OFF[m][1], c = k + NB_OFF[m][2];
                    double cm = K->c[m >> 1];
                    int kind = nb_kind(K, a, b, c);
                    if (kind == 0) {
                        d += cm;
                        s -= cm * x[NODE(g, a, b, c)];
                    } else if (kind == 1) {
                        d += cm;
                    }
                }
                y[u] = d * x[u] + s;
                if (diag) diag[u] = d;
            }
}

int eo_newton_pcg(const eo_grid *g, double *phi, const double *rho, const int *obj,
                  const int *target, double phi0, double te0, double n0, int nr_max, double nr_tol,
                  int pcg_max, double pcg_tol, int *nr_it_out, int *pcg_it_out) {
    return eo_newton_pcg_fb(g, phi, rho, obj, target, phi0, te0, n0, nr_max, nr_tol, pcg_max, pcg_tol, 0, 0.0, 0,
                            nr_it_out, pcg_it_out, NULL);
}

/* Newton-PCG as above, with the reference's fallback when the linear PCG
 * fails (ch3/ver2/PotentialSolver.cpp:270-271): Gauss-Seidel with omega 1
 * (solveGSLinear, :433-461) on J y = F from the PCG's last iterate, in node
 * order, its residual's RMS over all nodes checked at sweeps 0, 25, 50, ...
 * against gs_tol, at most gs_max sweeps (0: no fallback).  With early_stop
 * the inner PCG also stops, as the CUDA path's does, once the RMS of the
 * preconditioned residual z (over all nodes) is below nr_tol / 2, and z
 * itself is the update when the first z already is. */
int eo_newton_pcg_fb(const eo_grid *g, double *phi, const double *rho, const int *obj,
                     const int *target, double phi0, double te0, double n0, int nr_max, double nr_tol,
                     int pcg_max, double pcg_tol, int gs_max, double gs_tol, int early_stop, int *nr_it_out,
                     int *pcg_it_out, int *gs_it_out) {
    int gs_total = 0;
    int64_t nn = (int64_t)g->ni * g->nj * g->nk;
    nk_ctx K = {g, obj, {1.0 / (g->dh[0] * g->dh[0]), 1.0 / (g->dh[1] * g->dh[1]),
                         1.0 / (g->dh[2] * g->dh[2])}};
    double *bD = calloc(nn, sizeof(double)), *F = calloc(nn, sizeof(double));
    double *diagL = calloc(nn, sizeof(double)), *Pd = calloc(nn, sizeof(double));
    double *y = calloc(nn, sizeof(double)), *r = calloc(nn, sizeof(double));
    double *z = calloc(nn, sizeof(double)), *p = calloc(nn, sizeof(double));
    double *q = calloc(nn, sizeof(double)), *xu = calloc(nn, sizeof(double));
    /* Dirichlet contributions */
    for (int k = 1; k < g->nk - 1; k++)
        for (int j = 1; j < g->nj - 1; j++)
            for (int i = 1; i < g->ni - 1; i++) {
                int64_t u = NODE(g, i, j, k);
                if (obj[u] != 0) continue;
                double s = 0;
                for (int m = 0; m < 6; m++) {
                    int a = i + NB_OFF[m][0], b = j + NB_OFF[m][1], c = k + NB_OFF[m][2];
                    if (nb_kind(&K, a, b, c) == 1) s += K.c[m >> 1] * phi[NODE(g, a, b, c)];
                }
                bD[u] = s;
            }
    const double A0 = EO_QE * n0 / EO_EPS_0;
    int conv = 0, nr, pcg_total = 0;
    for (nr = 0; nr < nr_max; nr++) {
        for (int64_t u = 0; u < nn; u++) xu[u] = (obj[u] == 0) ? phi[u] : 0;
        apply_L(&K, xu, F, diagL);
        double fn = 0;
        for (int k = 1; k < g->nk - 1; k++)
            for (int j = 1; j < g->nj - 1; j++)
                for (int i = 1; i < g->ni - 1; i++) {
                    int64_t u = NODE(g, i, j, k);
                    if (obj[u] != 0) continue;
                    double e = exp((phi[u] - phi0) / te0);
                    F[u] = F[u] - bD[u] + A0 * e - rho[u] / EO_EPS_0;
                    Pd[u] = A0 / te0 * e;
                    fn += F[u] * F[u];
                }
        /* PCG on J y = F from y = 0 */
        double rz = 0;
        for (int64_t u = 0; u < nn; u++) {
            y[u] = 0;
            r[u] = F[u];
            double dg = diagL[u] + Pd[u];
            z[u] = (dg != 0) ? r[u] / dg : 0;
            p[u] = z[u];
            rz += r[u] * z[u];
        }
        double stop2 = pcg_tol * pcg_tol * fn;
        const double zz_stop = nr_tol * nr_tol / 4.0 * (double)nn;
        int it = 0, pcg_ok = 0, take_z = 0;
        if (early_stop && fn > 0) {
            double zz = 0;
            for (int64_t u = 0; u < nn; u++) zz += z[u] * z[u];
            if (zz < zz_stop) {
                take_z = 1;
                pcg_ok = 1;
                for (int64_t u = 0; u < nn; u++) y[u] = z[u];
            }
        }
        if (fn > 0 && !take_z) {
            for (it = 0; it < pcg_max; it++) {
                apply_L(&K, p, q, NULL);
                double pq = 0;
                for (int64_t u = 0; u < nn; u++) {
                    q[u] += Pd[u] * p[u];
                    pq += p[u] * q[u];
                }
                double alpha = rz / pq;
                double rr = 0;
                for (int64_t u = 0; u < nn; u++) {
                    y[u] += alpha * p[u];
                    r[u] -= alpha * q[u];
                    rr += r[u] * r[u];
                }
                if (rr <= stop2) {
                    it++;
                    pcg_ok = 1;
                    break;
                }
                double rz_new = 0, zz = 0;
                for (int64_t u = 0; u < nn; u++) {
                    double dg = diagL[u] + Pd[u];
                    z[u] = (dg != 0) ? r[u] / dg : 0;
                    rz_new += r[u] * z[u];
                    zz += z[u] * z[u];
                }
                if (early_stop && zz < zz_stop) {
                    it++;
                    pcg_ok = 1;
                    break;
                }
                double beta = rz_new / rz;
                rz = rz_new;
                for (int64_t u = 0; u < nn; u++) p[u] = z[u] + beta * p[u];
            }
        }
        pcg_total += it;
        if (fn > 0 && !pcg_ok && gs_max > 0) {
            /* Gauss-Seidel on J y = F from the PCG's y, in node order */
            for (int sw = 0; sw < gs_max; sw++) {
                for (int k = 1; k < g->nk - 1; k++)
                    for (int j = 1; j < g->nj - 1; j++)
                        for (int i = 1; i < g->ni - 1; i++) {
                            int64_t u = NODE(g, i, j, k);
                            if (obj[u] != 0) continue;
                            double s = F[u];
                            for (int m = 0; m < 6; m++) {
                                int a = i + NB_OFF[m][0], b = j + NB_OFF[m][1], c = k + NB_OFF[m][2];
                                if (nb_kind(&K, a, b, c) == 0) s += K.c[m >> 1] * y[NODE(g, a, b, c)];
                            }
                            y[u] = s / (diagL[u] + Pd[u]);
                        }
                gs_total++;
                if (sw % 25 == 0) {
                    apply_L(&K, y, q, NULL);
                    double R2 = 0;
                    for (int64_t u = 0; u < nn; u++) {
                        if (obj[u] != 0) continue;
                        double R = q[u] + Pd[u] * y[u] - F[u];
                        R2 += R * R;
                    }
                    if (sqrt(R2 / nn) < gs_tol) break;
                }
            }
        }
        double yn = 0;
        for (int64_t u = 0; u < nn; u++) {
            if (obj[u] != 0) continue;
            phi[u] -= y[u];
            yn += y[u] * y[u];
        }
        double norm = sqrt(yn / nn);
        if (norm < nr_tol) {
            conv = 1;
            nr++;
            break;
        }
    }
    for (int64_t u = 0; u < nn; u++)
        if (target[u] >= 0) phi[u] = phi[target[u]];
    free(bD);
    free(F);
    free(diagL);
    free(Pd);
    free(y);
    free(r);
    free(z);
    free(p);
    free(q);
    free(xu);
    if (nr_it_out) *nr_it_out = nr;
    if (pcg_it_out) *pcg_it_out = pcg_total;
    if (gs_it_out) *gs_it_out = gs_total;
    return conv;
}

/* PotentialSolver::computeEF, ch2/PotentialSolver.cpp:70-110 (identical in
 * ch3/ver2/PotentialSolver.cpp:465-504). */
void eo_efield(const eo_grid *g, const double *phi, double *ef) {
    double dx = g->dh[0], dy = g->dh[1], dz = g->dh[2];
    int64_t sy = g->ni, sz = (int64_t)g->ni * g->nj;
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++)
            for (int k = 0; k < g->nk; k++) {
                int64_t u = NODE(g, i, j, k);
                double *e = ef + 3 * u;
                if (i == 0)
                    e[0] = -(-3 * phi[u] + 4 * phi[u + 1] - phi[u + 2]) / (2 * dx);
                else if (i == g->ni - 1)
                    e[0] = -(phi[u - 2] - 4 * phi[u - 1] + 3 * phi[u]) / (2 * dx);
                else
                    e[0] = -(phi[u + 1] - phi[u - 1]) / (2 * dx);
                if (j == 0)
                    e[1] = -(-3 * phi[u] + 4 * phi[u + sy] - phi[u + 2 * sy]) / (2 * dy);
                else if (j == g->nj - 1)
                    e[1] = -(phi[u - 2 * sy] - 4 * phi[u - sy] + 3 * phi[u]) / (2 * dy);
                else
                    e[1] = -(phi[u + sy] - phi[u - sy]) / (2 * dy);
                if (k == 0)
                    e[2] = -(-3 * phi[u] + 4 * phi[u + sz] - phi[u + 2 * sz]) / (2 * dz);
                else if (k == g->nk - 1)
                    e[2] = -(phi[u - 2 * sz] - 4 * phi[u - sz] + 3 * phi[u]) / (2 * dz);
                else
                    e[2] = -(phi[u + sz] - phi[u - sz]) / (2 * dz);
            }
}

/* Species::getRealCount / getMomentum / getKE, ch2/Species.cpp:144-168.
 * out = {real count, px, py, pz, KE}. */
void eo_species_diag(const double *P, int64_t stride, int64_t n, double mass, double out[5]) {
    double cnt = 0, m[3] = {0, 0, 0}, ke = 0;
    for (int64_t p = 0; p < n; p++) {
        double w = P[6 * stride + p];
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        cnt += w;
        for (int d = 0; d < 3; d++) m[d] += v[d] * w;
        double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        ke += w * v2;
    }
    out[0] = cnt;
    for (int d = 0; d < 3; d++) out[1 + d] = m[d] * mass;
    out[4] = 0.5 * mass * ke;
}

/* World::getPE, ch2/World.cpp:72-84 */
double eo_potential_energy(const eo_grid *g, const double *ef, const double *vol) {
    double pe = 0;
    for (int i = 0; i < g->ni; i++)
        for (int j = 0; j < g->nj; j++)
            for (int k = 0; k < g->nk; k++) {
                int64_t u = NODE(g, i, j, k);
                const double *e = ef + 3 * u;
                double ef2 = e[0] * e[0] + e[1] * e[1] + e[2] * e[2];
                pe += ef2 * vol[u];
            }
    return 0.5 * EO_EPS_0 * pe;
}

/* Field_::updateAverage, ch3/ver2/Field.h:214-220 */
void eo_update_average(int64_t nn, double *ave, const double *inst, int samples) {
    for (int64_t u = 0; u < nn; u++) ave[u] = (inst[u] + samples * ave[u]) / (samples + 1);
}

/* ------------------------------------------------------------------------ */
/* ch4 species moments.  Species::sampleMoments, ch4/Species.cpp:191-201:
 * n_sum += mpw, nv_sum += mpw vel, nuu_sum += (mpw u) u, ... each with
 * Field_::scatter (ch4/Field.h:212-232; a double3 value scatters per
 * component), float64 sums in particle order.  mom: 7 planes of nn (n, nu,
 * nv, nw, nuu, nvv, nww). */
void eo_sample_moments(const eo_grid *g, const double *P, int64_t stride, int64_t n, double *mom) {
    const int64_t nn = (int64_t)g->ni * g->nj * g->nk;
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double lc[3], f[3], w[8];
        int c[3];
        int64_t idx[8];
        eo_xtol(g, x, lc);
        cell_of(g, lc, c, f);
        cic_nodes(g, c, idx);
        const double mpw = P[6 * stride + p], u = P[3 * stride + p], v = P[4 * stride + p], ww = P[5 * stride + p];
        const double val[7] = {mpw, mpw * u, mpw * v, mpw * ww, mpw * u * u, mpw * v * v, mpw * ww * ww};
        for (int q = 0; q < 7; q++) {
            cic_weights(val[q], f[0], f[1], f[2], w);
            for (int m = 0; m < 8; m++) mom[q * nn + idx[m]] += w[m];
        }
    }
}

/* Species::computeGasProperties, ch4/Species.cpp:204-225: vel = nv/n (0 where
 * n == 0, Field_ operator/ ch4/Field.h:182-196), T = m/(2K) (uu + vv + ww)
 * with uu = nuu/n - u u (T = 0 where n <= 0).  vel: [nn][3]. */
void eo_gas_properties(const eo_grid *g, double mass, const double *mom, double *vel, double *T) {
    const double K = 1.380648e-23;
    const int64_t nn = (int64_t)g->ni * g->nj * g->nk;
    for (int64_t u = 0; u < nn; u++) {
        const double count = mom[u];
        double ave[3];
        for (int d = 0; d < 3; d++) {
            ave[d] = count != 0 ? mom[(1 + d) * nn + u] / count : 0.0;
            vel[3 * u + d] = ave[d];
        }
        if (count <= 0) {
            T[u] = 0;
            continue;
        }
        const double uu = mom[4 * nn + u] / count - ave[0] * ave[0];
        const double vv = mom[5 * nn + u] / count - ave[1] * ave[1];
        const double ww = mom[6 * nn + u] / count - ave[2] * ave[2];
        T[u] = mass / (2 * K) * (uu + vv + ww);
    }
}

/* Species::computeMPC, ch4/Species.cpp:228-235: particles per cell by
 * World::XtoIJK (ch4/World.h:88-92); mpc[(k (nj-1) + j) (ni-1) + i] */
void eo_compute_mpc(const eo_grid *g, const double *P, int64_t stride, int64_t n, double *mpc) {
    const int64_t n_cells = (int64_t)(g->ni - 1) * (g->nj - 1) * (g->nk - 1);
    for (int64_t c = 0; c < n_cells; c++) mpc[c] = 0;
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]}, lc[3];
        eo_xtol(g, x, lc);
        const int i = (int)lc[0], j = (int)lc[1], k = (int)lc[2];
        mpc[((int64_t)k * (g->nj - 1) + j) * (g->ni - 1) + i] += 1;
    }
}

/* Field_<double>::gather, ch4/Field.h:234-253, with the index clamp */
static double gather1(const eo_grid *g, const double *f, const double lc[3]) {
    int c[3];
    double fr[3];
    int64_t idx[8];
    cell_of(g, lc, c, fr);
    cic_nodes(g, c, idx);
    const double di = fr[0], dj = fr[1], dk = fr[2];
    return f[idx[0]] * (1 - di) * (1 - dj) * (1 - dk) + f[idx[1]] * (di) * (1 - dj) * (1 - dk) +
           f[idx[2]] * (di) * (dj) * (1 - dk) + f[idx[3]] * (1 - di) * (dj) * (1 - dk) +
           f[idx[4]] * (1 - di) * (1 - dj) * (dk) + f[idx[5]] * (di) * (1 - dj) * (dk) +
           f[idx[6]] * (di) * (dj) * (dk) + f[idx[7]] * (1 - di) * (dj) * (dk);
}

/* MCC_CEX::apply, ch4/Collisions.cpp:43-80: for each source particle in
 * order, vt = target vel gathered, nn = target den gathered, P = 1 -
 * exp(-nn sigma |v - vt| dt) with sigma = 1e-16; one rnd() per particle and,
 * on a collision (P >= rnd()), the 11 of target.sampleIsotropicVel
 * (ch4/Species.cpp:149-174: theta, r, then 9 in sampleVth), whose velocity
 * the reference discards; the particle's velocity becomes 0.  p_off[p]: the
 * index in u of particle p's uniform.  Returns the collisions. */
int64_t eo_mcc_cex(const eo_grid *g, double *P, int64_t stride, int64_t n, const double *den, const double *vel,
                   double dt, const double *u, int64_t nu, int64_t *u_used, int64_t *p_off) {
    int64_t k = 0, ncol = 0;
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]}, lc[3], vt[3], vr[3];
        eo_xtol(g, x, lc);
        eo_gather3(g, vel, lc, vt);
        const double nn = gather1(g, den, lc);
        for (int d = 0; d < 3; d++) vr[d] = P[(3 + d) * stride + p] - vt[d];
        const double v_rel_mag = dsmc_mag(vr);
        const double sigma = 1e-16;
        const double Pc = 1 - exp(-nn * sigma * v_rel_mag * dt);
        if (p_off) p_off[p] = k;
        const double U = k < nu ? u[k] : -1.0;
        k++;
        if (Pc >= U) {
            k += 11;
            ncol++;
            for (int d = 0; d < 3; d++) P[(3 + d) * stride + p] = 0;
        }
    }
    if (u_used) *u_used = k;
    return ncol;
}

/* ------------------------------------------------------------------------ */
/* ch4 neutral push: Species::advance(neutrals, spherium) for a species of
 * charge 0, ch4/Species.cpp:8-91.  Each particle carries its own time left
 * (pdt, ch4/Species.h:15): the step adds the world's dt, the particle moves
 * for its whole time, leaves the domain (killed), or hits the sphere: it is
 * put 0.999 of the way to the intersection (World::lineSphereIntersect,
 * ch4/World.cpp:160-182), its time becomes the time used so far, and it
 * leaves with the thermal speed of a 1000 K wall in a diffuse direction
 * (Species::sampleReflectedVelocity, ch4/Species.cpp:94-100;
 * World::sphereDiffuseVector, ch4/World.cpp:185-199), then moves again.
 * The E-field kick is q/m E dt = 0 for a neutral and is left out.  Dead
 * particles are removed by swap-with-last (ch4/Species.cpp:76-89).
 * u: 11 uniforms per bounce (9 of sampleVth(1000), then sin_theta and psi);
 * p_off[p] (may be NULL): the index in u of particle p's first uniform.
 * sphere: centre and radius^2.  holes != 0 removes the dead in the CUDA
 * path's order instead.  Returns the particle count after removal; -1 when u
 * runs out. */
static double dot3(const double a[3], const double b[3]) {
    double s = 0;
    for (int i = 0; i < 3; i++) s += a[i] * b[i];
    return s;
}

static void cross3(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

static double line_sphere(const double sphere[4], const double x1[3], const double x2[3]) {
    double B[3], A[3];
    for (int i = 0; i < 3; i++) {
        B[i] = x2[i] - x1[i];
        A[i] = x1[i] - sphere[i];
    }
    const double a = dot3(B, B), b = 2 * dot3(A, B), c = dot3(A, A) - sphere[3];
    const double det = b * b - 4 * a * c;
    if (det < 0) return 0.5;
    double tp = (-b + sqrt(det)) / (2 * a);
    if (tp < 0 || tp > 1.0) {
        tp = (-b - sqrt(det)) / (2 * a);
        if (tp < 0 || tp > 1.0) tp = 0.5;
    }
    return tp;
}

static int in_sphere_ch4(const double sphere[4], const double x[3]) {
    double r[3] = {x[0] - sphere[0], x[1] - sphere[1], x[2] - sphere[2]};
    return (r[0] * r[0] + r[1] * r[1] + r[2] * r[2]) <= sphere[3];
}

/* sampleVth(T) (ch4/Species.cpp:149-158) from 9 uniforms */
static double sample_vth(double mass, double temp, const double *u) {
    double v_th = sqrt(2 * EO_K * temp / mass);
    double v1 = v_th * (u[0] + u[1] + u[2] - 1.5);
    double v2 = v_th * (u[3] + u[4] + u[5] - 1.5);
    double v3 = v_th * (u[6] + u[7] + u[8] - 1.5);
    return 3 / sqrt(2 + 2 + 2) * sqrt(v1 * v1 + v2 * v2 + v3 * v3);
}

/* sampleReflectedVelocity(pos, v_mag1) with sphereDiffuseVector(pos) */
static void reflect_diffuse(const double sphere[4], double mass, const double x[3], double v_mag1,
                            const double *u, double vel[3]) {
    const double v_th = sample_vth(mass, 1000, u);
    const double a_th = 1;
    const double v_mag2 = v_mag1 + a_th * (v_th - v_mag1);
    const double sin_theta = u[9];
    const double cos_theta = sqrt(1 - sin_theta * sin_theta);
    const double psi = 2 * EO_PI * u[10];
    double r[3] = {x[0] - sphere[0], x[1] - sphere[1], x[2] - sphere[2]}, n[3], t1[3], t2[3];
    const double m = sqrt(dot3(r, r));
    for (int i = 0; i < 3; i++) n[i] = r[i] / m;
    const double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0};
    if (dot3(n, ex) != 0)
        cross3(n, ex, t1);
    else
        cross3(n, ey, t1);
    cross3(n, t1, t2);
    for (int i = 0; i < 3; i++)
        vel[i] = v_mag2 * (sin_theta * cos(psi) * t1[i] + sin_theta * sin(psi) * t2[i] + cos_theta * n[i]);
}

int64_t eo_advance_ch4_neutral(const eo_grid *g, const double sphere[4], double mass, double dt, double *P,
                               int64_t stride, int64_t n, double *pdt, const double *u, int64_t nu,
                               int64_t *u_used, int64_t *p_off, int holes) {
    int64_t k = 0;
    for (int64_t p = 0; p < n; p++) {
        if (p_off) p_off[p] = k;
        pdt[p] += dt;
        int n_bounces = 0;
        while (pdt[p] > 0 && P[6 * stride + p] > 0) {
            double old[3], x[3], v[3];
            for (int i = 0; i < 3; i++) {
                old[i] = P[i * stride + p];
                v[i] = P[(3 + i) * stride + p];
                x[i] = old[i] + v[i] * pdt[p];
                P[i * stride + p] = x[i];
            }
            if (!eo_in_bounds(g, x)) {
                P[6 * stride + p] = 0;
            } else if (in_sphere_ch4(sphere, x)) {
                const double tp = line_sphere(sphere, old, x);
                const double dt_rem = (1 - tp) * pdt[p];
                pdt[p] -= dt_rem;
                const double s = 0.999 * tp;
                for (int i = 0; i < 3; i++) {
                    x[i] = old[i] + s * (x[i] - old[i]);
                    P[i * stride + p] = x[i];
                }
                const double v_mag1 = sqrt(dot3(v, v));
                if (k + 11 > nu) return -1;
                reflect_diffuse(sphere, mass, x, v_mag1, u + k, v);
                k += 11;
                for (int i = 0; i < 3; i++) P[(3 + i) * stride + p] = v[i];
                continue;
            }
            pdt[p] = 0;
            if (++n_bounces > 20) P[6 * stride + p] = 0;
        }
    }
    if (u_used) *u_used = k;
    if (holes) {
        /* the CUDA path's order: the r-th dead slot below the new count takes
         * the r-th live particle at or above it */
        int64_t alive = 0;
        for (int64_t p = 0; p < n; p++) alive += P[6 * stride + p] > 0;
        int64_t hole = 0;
        for (int64_t src = alive; src < n; src++) {
            if (!(P[6 * stride + src] > 0)) continue;
            while (P[6 * stride + hole] > 0) hole++;
            copy_particle(P, stride, hole, src);
            pdt[hole] = pdt[src];
            hole++;
        }
        return alive;
    }
    /* removal: a dead slot takes the last particle and is checked again */
    int64_t np = n;
    for (int64_t p = 0; p < np; p++) {
        if (P[6 * stride + p] > 0) continue;
        copy_particle(P, stride, p, np - 1);
        pdt[p] = pdt[np - 1];
        np--;
        p--;
    }
    return np;
}

/* ch4 ion push: Species::advance(neutrals, spherium) for a charged species,
 * ch4/Species.cpp:8-91.  The E kick uses the particle's whole time left
 * (v += E (dt q / m)); a particle leaving the domain is killed; one landing
 * in the sphere is put 0.999 of the way to the intersection and killed, and
 * creates (int)(mpw0 / neutral mpw0 + U) neutrals and, above 5000 m/s,
 * (int)(0.1 mpw0 / spherium mpw0 + U) sputtered particles, each with the
 * diffusely reflected velocity of sampleReflectedVelocity (the ion's mass in
 * sampleVth) through Species::addParticle (ch4/Species.cpp:103-119: rejected
 * outside the domain, velocity rewound by the target's q/m E dt/2, one dt
 * of time left).  New particles go to Q [7][max_new] in creation order with
 * tag 0 (neutral) or 1 (spherium), their time left in qdt.  Uniform order
 * per strike: the neutral count, 11 per neutral, the sputter count, 11 per
 * sputtered particle.  Returns the ion count after swap-with-last removal;
 * -1 when u runs out, -2 when Q is full. */
int64_t eo_advance_ch4_ion(const eo_grid *g, const double *ef, const double sphere[4], double charge, double mass,
                           double mpw0, double dt, double *P, int64_t stride, int64_t n, double *pdt,
                           double neu_mpw0, double neu_charge, double neu_mass, double sph_mpw0, double sph_charge,
                           double sph_mass, double *Q, int64_t max_new, int32_t *tag, double *qdt, int64_t *n_new,
                           const double *u, int64_t nu, int64_t *u_used) {
    return eo_advance_ch4_ion_ex(g, ef, sphere, charge, mass, mpw0, dt, P, stride, n, pdt, neu_mpw0, neu_charge,
                                 neu_mass, sph_mpw0, sph_charge, sph_mass, Q, max_new, tag, qdt, n_new, u, nu, u_used,
                                 NULL, 0);
}

/* as eo_advance_ch4_ion; p_off (optional, [n]) receives the index of each
 * particle's first uniform, and with holes the dead are removed in the CUDA
 * path's order (eo_compact_holes) instead of the reference's swap-with-last */
int64_t eo_advance_ch4_ion_ex(const eo_grid *g, const double *ef, const double sphere[4], double charge, double mass,
                              double mpw0, double dt, double *P, int64_t stride, int64_t n, double *pdt,
                              double neu_mpw0, double neu_charge, double neu_mass, double sph_mpw0, double sph_charge,
                              double sph_mass, double *Q, int64_t max_new, int32_t *tag, double *qdt, int64_t *n_new,
                              const double *u, int64_t nu, int64_t *u_used, int64_t *p_off, int holes) {
    int64_t k = 0, m = 0;
    for (int64_t p = 0; p < n; p++) {
        if (p_off) p_off[p] = k;
        pdt[p] += dt;
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]}, lc[3], e[3];
        eo_xtol(g, x, lc);
        eo_gather3(g, ef, lc, e);
        const double s = pdt[p] * charge / mass;
        for (int i = 0; i < 3; i++) P[(3 + i) * stride + p] += e[i] * s;
        int n_bounces = 0;
        while (pdt[p] > 0 && P[6 * stride + p] > 0) {
            double old[3], v[3];
            for (int i = 0; i < 3; i++) {
                old[i] = P[i * stride + p];
                v[i] = P[(3 + i) * stride + p];
                x[i] = old[i] + v[i] * pdt[p];
                P[i * stride + p] = x[i];
            }
            if (!eo_in_bounds(g, x)) {
                P[6 * stride + p] = 0;
            } else if (in_sphere_ch4(sphere, x)) {
                const double tp = line_sphere(sphere, old, x);
                const double dt_rem = (1 - tp) * pdt[p];
                pdt[p] -= dt_rem;
                const double sc = 0.999 * tp;
                for (int i = 0; i < 3; i++) {
                    x[i] = old[i] + sc * (x[i] - old[i]);
                    P[i * stride + p] = x[i];
                }
                const double v_mag1 = sqrt(dot3(v, v));
                P[6 * stride + p] = 0;
                for (int kind = 0; kind < 2; kind++) {
                    double ratio;
                    if (kind == 0) {
                        ratio = mpw0 / neu_mpw0;
                    } else {
                        const double sput_yield = (v_mag1 > 5000) ? 0.1 : 0;
                        ratio = sput_yield * mpw0 / sph_mpw0;
                    }
                    if (k >= nu) return -1;
                    const int create = (int)(ratio + u[k++]);
                    const double tq = kind == 0 ? neu_charge : sph_charge, tm = kind == 0 ? neu_mass : sph_mass;
                    const double tw = kind == 0 ? neu_mpw0 : sph_mpw0;
                    for (int c = 0; c < create; c++) {
                        if (k + 11 > nu) return -1;
                        double vel[3];
                        reflect_diffuse(sphere, mass, x, v_mag1, u + k, vel);
                        k += 11;
                        if (!eo_in_bounds(g, x)) continue;
                        if (m >= max_new) return -2;
                        double lc2[3], e2[3];
                        eo_xtol(g, x, lc2);
                        eo_gather3(g, ef, lc2, e2);
                        for (int i = 0; i < 3; i++) {
                            Q[i * max_new + m] = x[i];
                            Q[(3 + i) * max_new + m] = vel[i] - tq / tm * e2[i] * (0.5 * dt);
                        }
                        Q[6 * max_new + m] = tw;
                        tag[m] = kind;
                        qdt[m] = dt;
                        m++;
                    }
                }
                continue;
            }
            pdt[p] = 0;
            if (++n_bounces > 20) P[6 * stride + p] = 0;
        }
    }
    int64_t np = n;
    if (holes) {
        /* every survivor has used its time: pdt is 0 for all of them */
        np = eo_compact_holes(P, stride, n);
        for (int64_t p = 0; p < np; p++) pdt[p] = 0;
    } else {
        for (int64_t p = 0; p < np; p++) {
            if (P[6 * stride + p] > 0) continue;
            copy_particle(P, stride, p, np - 1);
            pdt[p] = pdt[np - 1];
            np--;
            p--;
        }
    }
    if (u_used) *u_used = k;
    if (n_new) *n_new = m;
    return np;
}

/* ChemistryIonize::apply, ch4/Collisions.cpp:10-31: over the cells (i
 * outer, then j, then k), n_a and n_e = rho / QE gathered at the cell centre,
 * dni = rate n_a n_e dt, and (int)(dni dV / mpw0 + U) ions are added.  Their
 * position is World::pos(i + U, j + U, k + U), which the overload taking
 * three ints (ch4/World.h:109-112) truncates to node (i, j, k); each is added
 * with addParticle(pos, 0, mpw0), whose third argument is the particle's
 * time left (ch4/Species.h:65-67): time mpw0, weight mpw0, velocity rewound
 * by q/m E dt/2 (ch4/Species.cpp:103-119).  Uniforms: one per cell, three per
 * ion.  New ions go to Q [7][max_new] with their time left in qdt; returns
 * their count, -1 when u runs out, -2 when Q is full. */
int64_t eo_chemistry_ionize(const eo_grid *g, const double *den_n, const double *rho, const double *ef,
                            double charge, double mass, double mpw0, double rate, double dt, double *Q,
                            int64_t max_new, double *qdt, const double *u, int64_t nu, int64_t *u_used) {
    return eo_chemistry_ionize_ex(g, den_n, rho, ef, charge, mass, mpw0, rate, dt, Q, max_new, qdt, u, nu, u_used,
                                  NULL);
}

/* as eo_chemistry_ionize; cell_off (optional, one entry per cell in the
 * reference's loop order, i outer, k inner) receives the index of each
 * cell's first uniform */
int64_t eo_chemistry_ionize_ex(const eo_grid *g, const double *den_n, const double *rho, const double *ef,
                               double charge, double mass, double mpw0, double rate, double dt, double *Q,
                               int64_t max_new, double *qdt, const double *u, int64_t nu, int64_t *u_used,
                               int64_t *cell_off) {
    const double QE_ = 1.602176565e-19;
    int64_t cidx = 0;
    const double dV = g->dh[0] * g->dh[1] * g->dh[2];
    int64_t k = 0, m = 0;
    for (int i = 0; i < g->ni - 1; i++)
        for (int j = 0; j < g->nj - 1; j++)
            for (int kk = 0; kk < g->nk - 1; kk++) {
                const double lc[3] = {i + 0.5, j + 0.5, kk + 0.5};
                const double na = gather1(g, den_n, lc);
                const double ne = gather1(g, rho, lc) / QE_;
                const double dni = rate * na * ne * dt;
                if (cell_off) cell_off[cidx] = k;
                cidx++;
                if (k >= nu) return -1;
                const int num_p = (int)(dni * dV / mpw0 + u[k++]);
                for (int p = 0; p < num_p; p++) {
                    if (k + 3 > nu) return -1;
                    k += 3;
                    const double x[3] = {g->x0[0] + g->dh[0] * (double)i, g->x0[1] + g->dh[1] * (double)j,
                                         g->x0[2] + g->dh[2] * (double)kk};
                    if (!eo_in_bounds(g, x)) continue;
                    if (m >= max_new) return -2;
                    double lc2[3], e[3];
                    eo_xtol(g, x, lc2);
                    eo_gather3(g, ef, lc2, e);
                    for (int d = 0; d < 3; d++) {
                        Q[d * max_new + m] = x[d];
                        Q[(3 + d) * max_new + m] = 0.0 - charge / mass * e[d] * (0.5 * dt);
                    }
                    Q[6 * max_new + m] = mpw0;
                    qdt[m] = mpw0;
                    m++;
                }
            }
    if (u_used) *u_used = k;
    return m;
}

/* ------------------------------------------------------------------------ */
/* Threaded CPU baseline: the per-thread particle ranges and private deposit
 * buffers of ch9/MT (Species.cpp:9-110), for the sphere push + compaction +
 * fixed-point deposit.  Returns seconds of wall time. */
#include <time.h>
typedef struct {
    const eo_grid *g;
    const double *ef;
    const double *sphere;
    double charge, mass, dt, fx;
    double *P;
    int64_t stride, p0, p1;
    int64_t *acc;
    int mode;
} bench_job;

static void *bench_worker(void *arg) {
    bench_job *J = (bench_job *)arg;
    if (J->mode == 0) {
        double *P = J->P;
        int64_t s = J->stride;
        /* push this range in place */
        double tmp_sph[4];
        memcpy(tmp_sph, J->sphere, sizeof tmp_sph);
        for (int64_t p = J->p0; p < J->p1; p++) {
            double q = J->dt * J->charge / J->mass;
            double x[3] = {P[p], P[s + p], P[2 * s + p]};
            double v[3] = {P[3 * s + p], P[4 * s + p], P[5 * s + p]};
            double lc[3], e[3];
            eo_xtol(J->g, x, lc);
            eo_gather3(J->g, J->ef, lc, e);
            for (int d = 0; d < 3; d++) v[d] += e[d] * q;
            for (int d = 0; d < 3; d++) x[d] += v[d] * J->dt;
            for (int d = 0; d < 3; d++) {
                P[d * s + p] = x[d];
                P[(3 + d) * s + p] = v[d];
            }
            if (in_sphere(tmp_sph, x) || !eo_in_bounds(J->g, x)) P[6 * s + p] = 0;
        }
    } else {
        eo_deposit_fixed(J->g, J->P + J->p0, J->stride, J->p1 - J->p0, J->fx, J->acc);
    }
    return NULL;
}

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

double eo_bench_push_deposit(const eo_grid *g, const double *ef, const double sphere[4],
                             double charge, double mass, double dt, double fx, double *P,
                             int64_t stride, int64_t n, int threads, int steps, int64_t *n_out,
                             int64_t *acc) {
    if (threads < 1) threads = 1;
    if (threads > 256) threads = 256;
    int64_t nn = (int64_t)g->ni * g->nj * g->nk;
    int64_t **bufs = calloc(threads, sizeof(int64_t *));
    for (int t = 0; t < threads; t++) bufs[t] = calloc(nn, sizeof(int64_t));
    pthread_t th[256];
    bench_job jobs[256];
    double t0 = now_s();
    for (int st = 0; st < steps; st++) {
        for (int mode = 0; mode < 2; mode++) {
            int64_t per = n / threads;
            for (int t = 0; t < threads; t++) {
                bench_job *J = &jobs[t];
                J->g = g;
                J->ef = ef;
                J->sphere = sphere;
                J->charge = charge;
                J->mass = mass;
                J->dt = dt;
                J->fx = fx;
                J->P = P;
                J->stride = stride;
                J->p0 = t * per;
                J->p1 = (t == threads - 1) ? n : (t + 1) * per;
                J->acc = bufs[t];
                J->mode = mode;
                if (mode == 1) memset(bufs[t], 0, nn * sizeof(int64_t));
                pthread_create(&th[t], NULL, bench_worker, J);
            }
            for (int t = 0; t < threads; t++) pthread_join(th[t], NULL);
            if (mode == 0) n = eo_compact_swap_last(P, stride, n);
        }
        for (int64_t u = 0; u < nn; u++) {
            int64_t s = 0;
            for (int t = 0; t < threads; t++) s += bufs[t][u];
            acc[u] = s;
        }
    }
    double el = now_s() - t0;
    for (int t = 0; t < threads; t++) free(bufs[t]);
    free(bufs);
    if (n_out) *n_out = n;
    return el;
}

/* ======================================================================
 * The mixed particle form (the chosen GPU form): an int32 cell key
 * i | j<<10 | k<<20, a float in-cell offset and a float velocity, with the
 * species weight mpw0.  These functions restate the GPU arithmetic
 * operation by operation (float products, fused multiply-adds where the GPU
 * code names them), so that the GPU's mixed state and its integer charge can
 * be checked bit for bit; the float64 functions above then bound the
 * distance of the mixed form from the reference.
 *
 * Reference behaviour restated in float: Species::advance
 * (ch3/ver2/Species.cpp:7-48, ch2/Species.cpp:7-38) with Field_::gather
 * (ch2/Field.h:186-208); Species::computeNumberDensity
 * (ch2/Species.cpp:41-52) with Field_::scatter (ch2/Field.h:164-183).
 * ====================================================================== */

void eo_mix_args_set(eo_mix_args *a, const eo_grid *g, double charge, double mass, double dt,
                     const double *sphere) {
    a->ni = g->ni;
    a->nj = g->nj;
    a->nk = g->nk;
    a->qmdt = (float)(charge / mass * dt);
    for (int d = 0; d < 3; d++) {
        a->dtdh[d] = (float)(dt / g->dh[d]);
        a->dh[d] = (float)g->dh[d];
        a->sx[d] = (float)(g->x0[d] - (sphere ? sphere[d] : 0.0));
    }
    a->r2 = sphere ? (float)sphere[3] : -1.f;
}

void eo_ef_to_f32(int64_t nn, const double *ef, float *ef4) {
    for (int64_t u = 0; u < nn; u++) {
        for (int d = 0; d < 3; d++) ef4[4 * u + d] = (float)ef[3 * u + d];
        ef4[4 * u + 3] = 0.f;
    }
}

/* float64 block -> mixed form: World::XtoL in float64 (ch2/World.h:72-78),
 * truncation, clamp to [0, n-2], offset rounded to float */
void eo_to_mixed(const eo_grid *g, const double *P, int64_t pstride, int64_t n, int32_t *cell, float *off,
                 float *vel, int64_t stride) {
    const int nmax[3] = {g->ni, g->nj, g->nk};
    for (int64_t p = 0; p < n; p++) {
        int c[3];
        for (int d = 0; d < 3; d++) {
            double lc = (P[d * pstride + p] - g->x0[d]) / g->dh[d];
            int i = (int)lc;
            if (i < 0) i = 0;
            if (i > nmax[d] - 2) i = nmax[d] - 2;
            c[d] = i;
            off[d * stride + p] = (float)(lc - i);
            vel[d * stride + p] = (float)P[(3 + d) * pstride + p];
        }
        cell[p] = c[0] | (c[1] << 10) | (c[2] << 20);
    }
}

static inline void mix_unpack(int32_t key, int *i, int *j, int *k) {
    *i = key & 1023;
    *j = (key >> 10) & 1023;
    *k = key >> 20;
}

/* the eight CIC corner weights in float, Field_::scatter's corner order */
static inline void mix_cic(float fx, float fy, float fz, float w[8]) {
    const float gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    w[0] = gx * gy * gz;
    w[1] = fx * gy * gz;
    w[2] = fx * fy * gz;
    w[3] = gx * fy * gz;
    w[4] = gx * gy * fz;
    w[5] = fx * gy * fz;
    w[6] = fx * fy * fz;
    w[7] = gx * fy * fz;
}

/* a coordinate moved by v*dtdh cells: new cell index, offset in [0,1) */
static inline int mix_advance_axis(int i, float *f, float v, float dtdh) {
    float x = fmaf(v, dtdh, *f);
    float fl = floorf(x);
    i += (int)fl;
    x -= fl;
    if (x >= 1.f) {
        x -= 1.f;
        i += 1;
    }
    *f = x;
    return i;
}

/* one mirror bounce (ch2/Species.cpp:32-36) in cell units */
static inline void mix_reflect_axis(int *i, float *f, float *v, int n) {
    float p = (float)*i + *f;
    const float top = (float)(n - 1);
    if (p < 0.f) {
        p = -p;
        *v = -*v;
    } else if (p >= top) {
        p = 2.f * top - p;
        *v = -*v;
    }
    int ii = (int)p;
    if (ii > n - 2) ii = n - 2;
    if (ii < 0) ii = 0;
    *i = ii;
    *f = p - (float)ii;
}

/* One push of n particles in the mixed form: E gathered from the float copy
 * ef4 ([nn][4]) with a chain of fused multiply-adds in corner order,
 * v = fma(E, q/m dt, v), x moved in cell units, then the walls: reflecting
 * (walls 0) or absorbing with the sphere (walls 1).  dead[p] marks particles
 * absorbed or made non-finite. */
void eo_push_mixed(const eo_mix_args *a, const float *ef4, int walls, int32_t *cell, float *off, float *vel,
                   int64_t stride, int64_t n, uint8_t *dead) {
    const int64_t sy = a->ni, sz = (int64_t)a->ni * a->nj;
    for (int64_t p = 0; p < n; p++) {
        int i, j, k;
        mix_unpack(cell[p], &i, &j, &k);
        float fx = off[p], fy = off[stride + p], fz = off[2 * stride + p];
        float vx = vel[p], vy = vel[stride + p], vz = vel[2 * stride + p];
        float w[8];
        mix_cic(fx, fy, fz, w);
        const int64_t n0 = ((int64_t)k * a->nj + j) * a->ni + i;
        const int64_t idx[8] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy, n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
        float e[3];
        for (int d = 0; d < 3; d++) {
            float s = w[0] * ef4[4 * idx[0] + d];
            for (int c = 1; c < 8; c++) s = fmaf(w[c], ef4[4 * idx[c] + d], s);
            e[d] = s;
        }
        vx = fmaf(e[0], a->qmdt, vx);
        vy = fmaf(e[1], a->qmdt, vy);
        vz = fmaf(e[2], a->qmdt, vz);
        i = mix_advance_axis(i, &fx, vx, a->dtdh[0]);
        j = mix_advance_axis(j, &fy, vy, a->dtdh[1]);
        k = mix_advance_axis(k, &fz, vz, a->dtdh[2]);
        int gone = 0;
        if (walls == 0) {
            mix_reflect_axis(&i, &fx, &vx, a->ni);
            mix_reflect_axis(&j, &fy, &vy, a->nj);
            mix_reflect_axis(&k, &fz, &vz, a->nk);
        } else {
            gone = i < 0 || i > a->ni - 2 || j < 0 || j > a->nj - 2 || k < 0 || k > a->nk - 2;
            if (!gone && a->r2 >= 0.f) {
                const float rx = fmaf((float)i + fx, a->dh[0], a->sx[0]);
                const float ry = fmaf((float)j + fy, a->dh[1], a->sx[1]);
                const float rz = fmaf((float)k + fz, a->dh[2], a->sx[2]);
                gone = fmaf(rz, rz, fmaf(ry, ry, rx * rx)) <= a->r2;
            }
        }
        if (!(isfinite(fx) && isfinite(fy) && isfinite(fz) && isfinite(vx) && isfinite(vy) && isfinite(vz))) {
            gone = 1;
            i = j = k = 0;
            fx = fy = fz = 0.f;
        }
        cell[p] = (i & 1023) | ((j & 1023) << 10) | (k << 20);
        off[p] = fx;
        off[stride + p] = fy;
        off[2 * stride + p] = fz;
        vel[p] = vx;
        vel[stride + p] = vy;
        vel[2 * stride + p] = vz;
        dead[p] = (uint8_t)gone;
    }
}

/* The removal of the GPU path in the mixed form: the r-th dead slot below
 * the new count receives the r-th live particle above it (the holes order
 * of eo_compact_holes).  Returns the new count. */
int64_t eo_compact_mixed(int32_t *cell, float *off, float *vel, int64_t stride, int64_t n, const uint8_t *dead) {
    int64_t alive = 0;
    for (int64_t p = 0; p < n; p++) alive += !dead[p];
    int64_t hole = 0;
    for (int64_t src = alive; src < n; src++) {
        if (dead[src]) continue;
        while (!dead[hole]) hole++;
        cell[hole] = cell[src];
        for (int d = 0; d < 3; d++) {
            off[d * stride + hole] = off[d * stride + src];
            vel[d * stride + hole] = vel[d * stride + src];
        }
        hole++;
    }
    return alive;
}

/* The mixed deposit: each corner weight w (float, in [0,1]) becomes
 * round-half-even(w * 2^23) counts of mpw0 * 2^-23, added to the node's
 * int64 sum (particles with skip[p] set deposit nothing; skip may be NULL). */
void eo_deposit_mixed(const eo_grid *g, const int32_t *cell, const float *off, int64_t stride, int64_t n,
                      const uint8_t *skip, int64_t *acc) {
    const int64_t sy = g->ni, sz = (int64_t)g->ni * g->nj;
    for (int64_t p = 0; p < n; p++) {
        if (skip && skip[p]) continue;
        int i, j, k;
        mix_unpack(cell[p], &i, &j, &k);
        float w[8];
        mix_cic(off[p], off[stride + p], off[2 * stride + p], w);
        const int64_t n0 = ((int64_t)k * g->nj + j) * g->ni + i;
        const int64_t idx[8] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy, n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
        for (int c = 0; c < 8; c++) acc[idx[c]] += (int64_t)(uint32_t)rintf(w[c] * 8388608.f);
    }
}

/* mixed form -> float64: x = x0 + (i + f) dh, the GPU's one fused
 * multiply-add; v widened */
void eo_from_mixed(const eo_grid *g, const int32_t *cell, const float *off, const float *vel, int64_t stride,
                   int64_t n, double mpw0, double *P, int64_t pstride) {
    for (int64_t p = 0; p < n; p++) {
        int c[3];
        mix_unpack(cell[p], &c[0], &c[1], &c[2]);
        for (int d = 0; d < 3; d++) {
            P[d * pstride + p] = fma((double)c[d] + (double)off[d * stride + p], g->dh[d], g->x0[d]);
            P[(3 + d) * pstride + p] = (double)vel[d * stride + p];
        }
        P[6 * pstride + p] = mpw0;
    }
}
