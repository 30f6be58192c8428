/*
 * ch4_push.h -- one particle's step of the ch4 neutral push
 * (Species::advance(neutrals, spherium) for a species of charge 0,
 * ch4/Species.cpp:8-100), host and device.  Included by k_fp64.cu (built
 * with -fmad=false, so every product and sum rounds as the reference's do).
 *
 * The particle moves for its whole time t; leaving the domain kills it
 * (World::inBounds, ch4/World.h:60-64); landing in the sphere
 * (World::inSphere, ch4/World.cpp:119-126) puts it 0.999 of the way to the
 * intersection (World::lineSphereIntersect, ch4/World.cpp:160-182), leaves it
 * the time it had used, and re-emits it with the speed of a 1000 K wall
 * (full accommodation) in a diffuse direction (sampleReflectedVelocity,
 * ch4/Species.cpp:94-100; World::sphereDiffuseVector,
 * ch4/World.cpp:185-199); then it moves again.  The E-field kick is
 * q/m E dt = 0 for a neutral and is left out.
 *
 * Each bounce draws 11 uniforms in the reference's rnd() order: 9 for
 * sampleVth(1000) (three sums of three), then sin_theta and psi.
 */
#pragma once

#include <math.h>

#ifndef __CUDACC__
#define __host__
#define __device__
#endif

namespace espic {

#define CH4_PI 3.141592653
#define CH4_K 1.380648e-23

struct Ch4Geo {
    double x0[3], xm[3];
    double sph[4]; /* centre, radius^2 (negative: no sphere) */
};

/* vec3 dot, ch4/Field.h:21-23: ((0 + a0 b0) + a1 b1) + a2 b2 */
__host__ __device__ inline double c4_dot(const double a[3], const double b[3]) {
    double s = 0;
    for (int i = 0; i < 3; i++) s += a[i] * b[i];
    return s;
}

/* vec3 cross, ch4/Field.h:32-34 */
__host__ __device__ inline void c4_cross(const double a[3], const double b[3], double o[3]) {
    o[0] = a[1] * b[2] - a[2] * b[1];
    o[1] = a[2] * b[0] - a[0] * b[2];
    o[2] = a[0] * b[1] - a[1] * b[0];
}

__host__ __device__ inline bool c4_in_bounds(const Ch4Geo &G, const double x[3]) {
    for (int i = 0; i < 3; i++)
        if (x[i] < G.x0[i] || x[i] >= G.xm[i]) return false;
    return true;
}

__host__ __device__ inline bool c4_in_sphere(const Ch4Geo &G, const double x[3]) {
    const double r0 = x[0] - G.sph[0], r1 = x[1] - G.sph[1], r2 = x[2] - G.sph[2];
    return (r0 * r0 + r1 * r1 + r2 * r2) <= G.sph[3];
}

/* parametric position of the first crossing of the segment x1 -> x2 with
 * the sphere (0.5 when none is found) */
__host__ __device__ inline double c4_line_sphere(const Ch4Geo &G, const double x1[3], const double x2[3]) {
    double B[3], A[3];
    for (int i = 0; i < 3; i++) {
        B[i] = x2[i] - x1[i];
        A[i] = x1[i] - G.sph[i];
    }
    const double a = c4_dot(B, B), b = 2 * c4_dot(A, B), c = c4_dot(A, A) - G.sph[3];
    const double det = b * b - 4 * a * c;
    if (det < 0) return 0.5;
    double tp = (-b + sqrt(det)) / (2 * a);
    if (tp < 0 || tp > 1.0) {
        tp = (-b - sqrt(det)) / (2 * a);
        if (tp < 0 || tp > 1.0) tp = 0.5;
    }
    return tp;
}

/* Species::sampleReflectedVelocity (ch4/Species.cpp:94-100): speed
 * v_mag1 + a_th (v_th - v_mag1) with a_th = 1 and v_th of sampleVth(1000)
 * for the striking particle's mass, direction World::sphereDiffuseVector
 * (ch4/World.cpp:185-199) at x.  Uniforms U(k) .. U(k + 10): 9 for
 * sampleVth (three sums of three, ch4/Species.cpp:149-158), then sin_theta
 * and psi. */
template <class UF>
__host__ __device__ inline void c4_reflect(const Ch4Geo &G, double mass, const double x[3], double v_mag1, UF &U,
                                           int k, double vel[3]) {
    const double v_th = sqrt(2 * CH4_K * 1000 / mass);
    const double v1 = v_th * (U(k) + U(k + 1) + U(k + 2) - 1.5);
    const double v2 = v_th * (U(k + 3) + U(k + 4) + U(k + 5) - 1.5);
    const double v3 = v_th * (U(k + 6) + U(k + 7) + U(k + 8) - 1.5);
    /* 3 / sqrt(2 + 2 + 2) in the reference: sqrt of the int 6 is sqrt(6.0)
     * on the host; in device code sqrt must be given a double (an int
     * argument made nvcc drop the rest of the caller's branch) */
    const double vth = 3.0 / sqrt(6.0) * sqrt(v1 * v1 + v2 * v2 + v3 * v3);
    const double a_th = 1;
    const double v_mag2 = v_mag1 + a_th * (vth - v_mag1);
    const double sin_theta = U(k + 9);
    const double cos_theta = sqrt(1 - sin_theta * sin_theta);
    const double psi = 2 * CH4_PI * U(k + 10);
    double r[3] = {x[0] - G.sph[0], x[1] - G.sph[1], x[2] - G.sph[2]}, n[3], t1[3], t2[3];
    const double m = sqrt(c4_dot(r, r));
    for (int i = 0; i < 3; i++) n[i] = r[i] / m;
    const double ex[3] = {1, 0, 0}, ey[3] = {0, 1, 0};
    if (c4_dot(n, ex) != 0)
        c4_cross(n, ex, t1);
    else
        c4_cross(n, ey, t1);
    c4_cross(n, t1, t2);
    const double cp = cos(psi), sp = sin(psi);
    for (int i = 0; i < 3; i++) vel[i] = v_mag2 * (sin_theta * cp * t1[i] + sin_theta * sp * t2[i] + cos_theta * n[i]);
}

/* The step of one particle: t its time for this step, x and v updated in
 * place.  U(k) returns the particle's k-th uniform of the step.  Returns
 * the number of bounces; alive becomes false when the particle leaves the
 * domain or bounces more than max_bounces times (the reference has no such
 * bound on the bounce loop; 64 bounces in one step do not occur). */
template <class UF>
__host__ __device__ inline int ch4_advance_one(const Ch4Geo &G, double mass, double t, double x[3], double v[3],
                                               UF &U, bool &alive, int max_bounces) {
    int bounces = 0, n_steps = 0;
    alive = true;
    while (t > 0 && alive) {
        double old[3];
        for (int i = 0; i < 3; i++) {
            old[i] = x[i];
            x[i] = old[i] + v[i] * t;
        }
        if (!c4_in_bounds(G, x)) {
            alive = false;
        } else if (c4_in_sphere(G, x)) {
            const double tp = c4_line_sphere(G, old, x);
            const double dt_rem = (1 - tp) * t;
            t -= dt_rem;
            const double s = 0.999 * tp;
            for (int i = 0; i < 3; i++) x[i] = old[i] + s * (x[i] - old[i]);
            const double v_mag1 = sqrt(c4_dot(v, v));
            c4_reflect(G, mass, x, v_mag1, U, 11 * bounces, v);
            if (++bounces > max_bounces) alive = false;
            continue;
        }
        t = 0;
        if (++n_steps > 20) alive = false;
    }
    return bounces;
}

/* The move of one ion of ch4's ion branch (Species::advance of a charged
 * species, ch4/Species.cpp:26-85) after its E kick: it moves for its whole
 * time t; leaving the domain kills it (returns 1); landing in the sphere
 * puts it 0.999 of the way to the intersection, sets v_mag1 to its speed
 * and kills it (returns 2: the caller creates the neutrals and sputtered
 * particles); else it survives (returns 0).  The reference's loop ends after
 * one pass in every case: a surviving ion has no time left and a killed one
 * no weight. */
__host__ __device__ inline int ch4_ion_move(const Ch4Geo &G, double t, double x[3], const double v[3],
                                            double &v_mag1) {
    if (!(t > 0)) return 0;
    double old[3];
    for (int i = 0; i < 3; i++) {
        old[i] = x[i];
        x[i] = old[i] + v[i] * t;
    }
    if (!c4_in_bounds(G, x)) return 1;
    if (c4_in_sphere(G, x)) {
        const double tp = c4_line_sphere(G, old, x);
        const double s = 0.999 * tp;
        for (int i = 0; i < 3; i++) x[i] = old[i] + s * (x[i] - old[i]);
        v_mag1 = sqrt(c4_dot(v, v));
        return 2;
    }
    return 0;
}

}  // namespace espic
