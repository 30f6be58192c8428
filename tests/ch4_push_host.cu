/* ch4_push_host.cu -- TEST INFRASTRUCTURE: the GPU path's per-particle ch4
 * push (ch4_advance_one in csrc/ch4_push.h) compiled as host code, so the
 * CPU suite can compare its arithmetic with the oracle's restatement.
 * Built by tests/test_ch4_push_host.py with nvcc into a temporary folder. */
#include <stdint.h>
#include "ch4_push.h"

using namespace espic;

struct HostUniforms {
    const double *u;
    int64_t base;
    double operator()(int k) { return u[base + k]; }
};

/* one step of n particles: P [7][stride] updated in place (no removal),
 * alive[p] set; returns the bounces */
extern "C" int64_t ch4_host_step(const double x0[3], const double xm[3], const double sph[4], double mass, double dt,
                                 double *P, int64_t stride, int64_t n, const double *pdt, const double *u,
                                 const int64_t *p_off, int32_t *alive_out) {
    Ch4Geo G;
    for (int d = 0; d < 3; d++) {
        G.x0[d] = x0[d];
        G.xm[d] = xm[d];
    }
    for (int d = 0; d < 4; d++) G.sph[d] = sph[d];
    int64_t total = 0;
    for (int64_t p = 0; p < n; p++) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        HostUniforms U{u, p_off[p]};
        bool alive = true;
        total += ch4_advance_one(G, mass, pdt[p] + dt, x, v, U, alive, 64);
        for (int d = 0; d < 3; d++) {
            P[d * stride + p] = x[d];
            P[(3 + d) * stride + p] = v[d];
        }
        alive_out[p] = alive ? 1 : 0;
    }
    return total;
}
