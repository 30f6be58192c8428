/*
 * adjoint.cu -- a differentiable form of the sphere run and its hand-written
 * adjoint (no reference counterpart: the reference has no gradients).
 *
 * Forward model, per step n (the loop of ch3/ver2/Main.cpp:50-72 for one ion
 * species without injection; x in metres, v the leapfrog half-step velocity,
 * w the macroparticle weight):
 *   E^n   = -grad phi^n                     (PotentialSolver::computeEF)
 *   v+    = v + (q/m) dt sum_c S_c(x) E^n_c  (Field_::gather + Species::advance)
 *   x+    = x + dt v+
 *   w+    = w a(x+)                          (absorption, made C1: see below)
 *   rho   = q sum_p w+ S(x+) / node_vol      (computeNumberDensity, charge)
 *   phi+  = Boltzmann-electron solve of rho  (the Newton-PCG of k_pcg.cu)
 * Absorption at the sphere and the domain faces is a smooth factor: a = 1
 * outside an absorbing layer of thickness delta just inside the sphere
 * surface and each face, 0 beyond it, 1 - 3t^2 + 2t^3 across it (t the depth
 * into the layer / delta).  A particle's weight is the product of the factors
 * it has met, so a particle that entered an absorber stays at weight 0; no
 * particle is removed.  delta -> 0 gives the reference's removal
 * (ch3/ver2/Species.cpp:26-33); delta > 0 makes the loss a C1 function of
 * every input, which central differences can check.
 *
 * Loss: alpha * field energy of phi^N (World::getPE) + beta * ions in the
 * wake box, sum_p w_p sum_{corners c with z_c in [z0, z1]} S_c(x_p) (the CIC
 * density integrated over the box's nodes).
 *
 * Backward: the exact adjoint of the discrete forward -- push, gather (its
 * transpose scatters the particle field adjoints to the nodes), CIC deposit
 * (its transpose gathers rho_bar / node_vol), the E stencil (applied as G^T
 * in gather form), the Neumann copies (folded into their targets), the
 * Dirichlet sphere nodes (which feed d loss / d phi_sphere) and the solve:
 * J lambda = phi_bar with J the symmetric Jacobian at phi^n, by the same
 * Newton-PCG kernel in its linear mode.  Forward states are checkpointed
 * every K steps; the backward recomputes each K-step segment from its
 * checkpoint.  Particle arithmetic runs in T = double or float (the FP32 and
 * FP64 adjoints); solves use float64 outer iterations either way.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>

#include <algorithm>
#include <vector>

#include "espic.h"
#include "espic_world.h"

int espic_internal_fail(int code, const char *msg);

namespace espic {

#define AD_EPS_0 8.85418782e-12

struct DiffGeo {
    int ni, nj, nk;
    double x0[3], inv_dh[3];
    double xmin[3], xmax[3]; /* domain */
    double c[3], R;          /* sphere; R < 0: none */
    double delta;            /* absorbing layer */
};

template <typename T>
struct Cic {
    int i[3];
    T f[3], df[3]; /* in-cell fraction and d f / d x (0 where clamped) */
};

template <typename T>
__device__ __forceinline__ void cic_locate(const DiffGeo &G, const T x[3], Cic<T> &c) {
    const int n[3] = {G.ni, G.nj, G.nk};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const T lc = (x[d] - (T)G.x0[d]) * (T)G.inv_dh[d];
        const T fl = floor(lc);
        int i = (int)fl;
        T f = lc - fl, df = (T)G.inv_dh[d];
        if (i < 0) {
            i = 0;
            f = 0;
            df = 0;
        } else if (i > n[d] - 2) {
            i = n[d] - 2;
            f = 1;
            df = 0;
        }
        c.i[d] = i;
        c.f[d] = f;
        c.df[d] = df;
    }
}

/* weight of corner q (bit 0: +x, bit 1: +y, bit 2: +z) and its gradient */
template <typename T>
__device__ __forceinline__ T cic_corner(const Cic<T> &c, int q, T grad[3]) {
    T s[3], ds[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const bool hi = (q >> d) & 1;
        s[d] = hi ? c.f[d] : (T)1 - c.f[d];
        ds[d] = hi ? c.df[d] : -c.df[d];
    }
    grad[0] = ds[0] * s[1] * s[2];
    grad[1] = s[0] * ds[1] * s[2];
    grad[2] = s[0] * s[1] * ds[2];
    return s[0] * s[1] * s[2];
}

__device__ __forceinline__ int64_t corner_node(const DiffGeo &G, const Cic<float> &c, int q) {
    return ((int64_t)(c.i[2] + ((q >> 2) & 1)) * G.nj + (c.i[1] + ((q >> 1) & 1))) * G.ni + (c.i[0] + (q & 1));
}
__device__ __forceinline__ int64_t corner_node(const DiffGeo &G, const Cic<double> &c, int q) {
    return ((int64_t)(c.i[2] + ((q >> 2) & 1)) * G.nj + (c.i[1] + ((q >> 1) & 1))) * G.ni + (c.i[0] + (q & 1));
}

/* C1 step: 1 for t <= 0, 0 for t >= 1, 1 - 3t^2 + 2t^3 between */
template <typename T>
__device__ __forceinline__ T keep(T t, T &dk) {
    if (t <= (T)0) {
        dk = 0;
        return 1;
    }
    if (t >= (T)1) {
        dk = 0;
        return 0;
    }
    dk = (T)6 * t * (t - (T)1);
    return (T)1 - t * t * ((T)3 - (T)2 * t);
}

/* absorption factor a(x) and its gradient */
template <typename T>
__device__ __forceinline__ T absorb(const DiffGeo &G, const T x[3], T ga[3]) {
    T k[7], dk[7], gt[7][3];
    const T id = (T)(1.0 / G.delta);
    int m = 0;
#pragma unroll
    for (int d = 0; d < 3; d++) {
        /* lower face: depth from the layer's inner edge */
        T t = (T)1 - (x[d] - (T)G.xmin[d]) * id;
        k[m] = keep(t, dk[m]);
        gt[m][0] = gt[m][1] = gt[m][2] = 0;
        gt[m][d] = -id;
        m++;
        t = (T)1 - ((T)G.xmax[d] - x[d]) * id;
        k[m] = keep(t, dk[m]);
        gt[m][0] = gt[m][1] = gt[m][2] = 0;
        gt[m][d] = id;
        m++;
    }
    if (G.R > 0) {
        const T r0 = x[0] - (T)G.c[0], r1 = x[1] - (T)G.c[1], r2 = x[2] - (T)G.c[2];
        const T r = sqrt(r0 * r0 + r1 * r1 + r2 * r2);
        const T t = ((T)G.R - r) * id;
        k[m] = keep(t, dk[m]);
        const T ir = r > (T)0 ? (T)1 / r : (T)0;
        gt[m][0] = -r0 * ir * id;
        gt[m][1] = -r1 * ir * id;
        gt[m][2] = -r2 * ir * id;
    } else {
        k[m] = 1;
        dk[m] = 0;
        gt[m][0] = gt[m][1] = gt[m][2] = 0;
    }
    T a = 1;
#pragma unroll
    for (int q = 0; q < 7; q++) a *= k[q];
    ga[0] = ga[1] = ga[2] = 0;
#pragma unroll
    for (int q = 0; q < 7; q++) {
        if (dk[q] == (T)0) continue;
        T o = dk[q];
#pragma unroll
        for (int r = 0; r < 7; r++)
            if (r != q) o *= k[r];
#pragma unroll
        for (int d = 0; d < 3; d++) ga[d] += o * gt[q][d];
    }
    return a;
}

/* particle rows: x, y, z, vx, vy, vz, w (stride n) */
template <typename T>
__global__ void k_ad_weights0(DiffGeo G, T *P, int64_t n, T w0) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    T x[3] = {P[p], P[n + p], P[2 * n + p]}, ga[3];
    P[6 * n + p] = w0 * absorb(G, x, ga);
}

/* one push: in -> out (out may equal in) */
template <typename T>
__global__ void k_ad_push(DiffGeo G, const double *__restrict__ ef, const T *in, T *out, int64_t n, T k_e, T dt) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    T x[3] = {in[p], in[n + p], in[2 * n + p]};
    T v[3] = {in[3 * n + p], in[4 * n + p], in[5 * n + p]};
    const T w = in[6 * n + p];
    Cic<T> c;
    cic_locate(G, x, c);
    T e[3] = {0, 0, 0};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        T gs[3];
        const T s = cic_corner(c, q, gs);
        const int64_t u = corner_node(G, c, q);
#pragma unroll
        for (int d = 0; d < 3; d++) e[d] += s * (T)ef[3 * u + d];
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        v[d] += k_e * e[d];
        x[d] += dt * v[d];
    }
    T ga[3];
    const T a = absorb(G, x, ga);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        out[d * n + p] = x[d];
        out[(3 + d) * n + p] = v[d];
    }
    out[6 * n + p] = w * a;
}

/* q w S deposited (float64 atomics); divided by the node volume after */
template <typename T>
__global__ void k_ad_deposit(DiffGeo G, const T *__restrict__ P, int64_t n, double q, double *rho) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const T w = P[6 * n + p];
    if (w == (T)0) return;
    T x[3] = {P[p], P[n + p], P[2 * n + p]};
    Cic<T> c;
    cic_locate(G, x, c);
#pragma unroll
    for (int qq = 0; qq < 8; qq++) {
        T gs[3];
        const T s = cic_corner(c, qq, gs);
        atomicAdd(rho + corner_node(G, c, qq), q * (double)(w * s));
    }
}

__global__ void k_ad_per_volume(int64_t nn, double *x, const double *__restrict__ vol) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u < nn) x[u] = vol[u] != 0 ? x[u] / vol[u] : 0.0;
}

/* phi = phi_s on the sphere's nodes (object id 1) */
__global__ void k_ad_set_sphere(int64_t nn, const int32_t *__restrict__ obj, double phi_s, double *phi) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u < nn && obj[u] == 1) phi[u] = phi_s;
}

constexpr int AD_BLOCKS = 256, AD_THREADS = 256;

__device__ __forceinline__ void ad_block_store(double v, double *out) {
    __shared__ double sh[AD_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < AD_THREADS / 32; k++) s += sh[k];
        out[blockIdx.x] = s;
    }
}

/* out[0] (+)= scale * sum of partials[0..AD_BLOCKS) in block order */
__global__ void k_ad_final(const double *__restrict__ partials, double scale, double *out, int accumulate) {
    if (threadIdx.x != 0) return;
    double s = 0;
    for (int b = 0; b < AD_BLOCKS; b++) s += partials[b];
    out[0] = accumulate ? out[0] + scale * s : scale * s;
}

/* the wake-box ions sum_p w B(x), B(x) = sum of corner weights on box nodes */
template <typename T>
__global__ void __launch_bounds__(AD_THREADS) k_ad_wake(DiffGeo G, const T *__restrict__ P, int64_t n,
                                                        const uint8_t *__restrict__ box, double *partials) {
    double acc = 0;
    for (int64_t p = (int64_t)blockIdx.x * AD_THREADS + threadIdx.x; p < n; p += (int64_t)AD_BLOCKS * AD_THREADS) {
        const T w = P[6 * n + p];
        if (w == (T)0) continue;
        T x[3] = {P[p], P[n + p], P[2 * n + p]};
        Cic<T> c;
        cic_locate(G, x, c);
        T b = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) {
            T gs[3];
            const T s = cic_corner(c, q, gs);
            if (box[corner_node(G, c, q)]) b += s;
        }
        acc += (double)(w * b);
    }
    ad_block_store(acc, partials);
}

/* terminal adjoints: xb = beta w grad B, wb = beta B, vb = 0 */
template <typename T>
__global__ void k_ad_terminal(DiffGeo G, const T *__restrict__ P, int64_t n, const uint8_t *__restrict__ box,
                              T beta, T *A) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    T x[3] = {P[p], P[n + p], P[2 * n + p]};
    const T w = P[6 * n + p];
    Cic<T> c;
    cic_locate(G, x, c);
    T b = 0, gb[3] = {0, 0, 0};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        T gs[3];
        const T s = cic_corner(c, q, gs);
        if (!box[corner_node(G, c, q)]) continue;
        b += s;
#pragma unroll
        for (int d = 0; d < 3; d++) gb[d] += gs[d];
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        A[d * n + p] = beta * w * gb[d];
        A[(3 + d) * n + p] = 0;
    }
    A[6 * n + p] = beta * b;
}

/* adjoint of the deposit at state P: wb += G_g(x), xb += w grad G_g(x), with
 * g = q rho_bar / node_vol per node */
template <typename T>
__global__ void k_ad_deposit_adj(DiffGeo G, const T *__restrict__ P, int64_t n, const double *__restrict__ g,
                                 T *A) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    T x[3] = {P[p], P[n + p], P[2 * n + p]};
    const T w = P[6 * n + p];
    Cic<T> c;
    cic_locate(G, x, c);
    T s_acc = 0, gx[3] = {0, 0, 0};
#pragma unroll
    for (int q = 0; q < 8; q++) {
        T gs[3];
        const T s = cic_corner(c, q, gs);
        const T gu = (T)g[corner_node(G, c, q)];
        s_acc += s * gu;
#pragma unroll
        for (int d = 0; d < 3; d++) gx[d] += gs[d] * gu;
    }
#pragma unroll
    for (int d = 0; d < 3; d++) A[d * n + p] += w * gx[d];
    A[6 * n + p] += s_acc;
}

/* adjoint of the step n -> n+1 (Pn: state n, Pn1: state n+1, ef: E^n):
 * weights, position, velocity, then the gather (its transpose scatters
 * Ebar) */
template <typename T>
__global__ void k_ad_step(DiffGeo G, const double *__restrict__ ef, const T *__restrict__ Pn,
                          const T *__restrict__ Pn1, int64_t n, T k_e, T dt, T *A, double *Ebar) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    T xb[3] = {A[p], A[n + p], A[2 * n + p]};
    T vb[3] = {A[3 * n + p], A[4 * n + p], A[5 * n + p]};
    T wb = A[6 * n + p];
    /* w+ = w a(x+) */
    {
        T x1[3] = {Pn1[p], Pn1[n + p], Pn1[2 * n + p]}, ga[3];
        const T a = absorb(G, x1, ga);
        const T wn = Pn[6 * n + p];
#pragma unroll
        for (int d = 0; d < 3; d++) xb[d] += wb * wn * ga[d];
        wb *= a;
    }
    /* x+ = x + dt v+ ; v+ = v + k E */
    T eb[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        vb[d] += dt * xb[d];
        eb[d] = k_e * vb[d];
    }
    /* gather at x^n */
    T x[3] = {Pn[p], Pn[n + p], Pn[2 * n + p]};
    Cic<T> c;
    cic_locate(G, x, c);
#pragma unroll
    for (int q = 0; q < 8; q++) {
        T gs[3];
        const T s = cic_corner(c, q, gs);
        const int64_t u = corner_node(G, c, q);
        const T ed = (T)ef[3 * u] * eb[0] + (T)ef[3 * u + 1] * eb[1] + (T)ef[3 * u + 2] * eb[2];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            xb[d] += gs[d] * ed;
            atomicAdd(Ebar + 3 * u + d, (double)(s * eb[d]));
        }
    }
#pragma unroll
    for (int d = 0; d < 3; d++) {
        A[d * n + p] = xb[d];
        A[(3 + d) * n + p] = vb[d];
    }
    A[6 * n + p] = wb;
}

/* xb += wb w0 grad a(x^0) (the initial weights) */
template <typename T>
__global__ void k_ad_initial(DiffGeo G, const T *__restrict__ P0, int64_t n, T w0, T *A) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    T x[3] = {P0[p], P0[n + p], P0[2 * n + p]}, ga[3];
    absorb(G, x, ga);
    const T wb = A[6 * n + p];
#pragma unroll
    for (int d = 0; d < 3; d++) A[d * n + p] += wb * w0 * ga[d];
}

/* Ebar = alpha eps0 vol E (the field-energy term) */
__global__ void k_ad_pe_adj(int64_t nn, const double *__restrict__ ef, const double *__restrict__ vol, double alpha,
                            double *Ebar) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    const double s = alpha * AD_EPS_0 * vol[u];
    for (int d = 0; d < 3; d++) Ebar[3 * u + d] = s * ef[3 * u + d];
}

/* phi_bar = G^T Ebar, G the E stencil of k_efield (E = -grad phi: central
 * differences inside, (-3, 4, -1) / 2h one-sided on the faces), in gather
 * form: node v collects every E component whose stencil contains it */
__device__ __forceinline__ double gradT_axis(const double *Eb, int64_t v, int iv, int nax, int64_t st, int comp,
                                             double inv2h) {
    double acc = 0;
    /* central stencils of the interior neighbours u = v -+ 1:
     * dE_u/dphi_{u+1} = -1/2h, dE_u/dphi_{u-1} = +1/2h */
    if (iv - 1 >= 1 && iv - 1 <= nax - 2) acc += Eb[3 * (v - st) + comp] * (-inv2h);
    if (iv + 1 >= 1 && iv + 1 <= nax - 2) acc += Eb[3 * (v + st) + comp] * inv2h;
    /* face u = 0: E = -(-3 phi0 + 4 phi1 - phi2) / 2h */
    if (iv <= 2) {
        const double cf = iv == 0 ? 3.0 : (iv == 1 ? -4.0 : 1.0);
        acc += Eb[3 * (v - (int64_t)iv * st) + comp] * cf * inv2h;
    }
    /* face u = n-1: E = -(phi_{n-3} - 4 phi_{n-2} + 3 phi_{n-1}) / 2h */
    if (iv >= nax - 3) {
        const int r = nax - 1 - iv;
        const double cf = r == 0 ? -3.0 : (r == 1 ? 4.0 : -1.0);
        acc += Eb[3 * (v + (int64_t)r * st) + comp] * cf * inv2h;
    }
    return acc;
}

__global__ void k_ad_gradT(Geo g, const double *__restrict__ Eb, double *phib) {
    int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (v >= nn) return;
    const int i = (int)(v % g.ni), j = (int)((v / g.ni) % g.nj), k = (int)(v / ((int64_t)g.ni * g.nj));
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    double acc = gradT_axis(Eb, v, i, g.ni, 1, 0, 1.0 / (2 * g.dh[0]));
    acc += gradT_axis(Eb, v, j, g.nj, sy, 1, 1.0 / (2 * g.dh[1]));
    acc += gradT_axis(Eb, v, k, g.nk, sz, 2, 1.0 / (2 * g.dh[2]));
    phib[v] = acc;
}

/* Neumann copies phi_b = phi_t: phi_bar_t += phi_bar_b */
__global__ void k_ad_fold(int64_t nn, const int32_t *__restrict__ target, double *phib) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    const int32_t t = target[u];
    if (t >= 0) {
        atomicAdd(phib + t, phib[u]);
        phib[u] = 0;
    }
}

/* partials of sum over sphere nodes of phi_bar (phi = phi_s there) */
__global__ void __launch_bounds__(AD_THREADS) k_ad_sphere_direct(int64_t nn, const int32_t *__restrict__ obj,
                                                                 const double *__restrict__ phib, double *partials) {
    double acc = 0;
    for (int64_t u = (int64_t)blockIdx.x * AD_THREADS + threadIdx.x; u < nn; u += (int64_t)AD_BLOCKS * AD_THREADS)
        if (obj[u] == 1) acc += phib[u];
    ad_block_store(acc, partials);
}

/* from lambda = J^-1 phi_bar: g = q lambda / (eps0 vol) on the unknowns
 * (rho_bar = lambda / eps0), and the partials of the sphere coupling
 * sum_u lambda_u sum_{sphere neighbours} c (dF_u / dphi_s = -sum c) */
__global__ void __launch_bounds__(AD_THREADS) k_ad_after_solve(Geo g, const int32_t *__restrict__ obj,
                                                               const double *__restrict__ lam,
                                                               const double *__restrict__ vol, double q, double *gn,
                                                               double *partials) {
    const int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    const double cd[3] = {1.0 / (g.dh[0] * g.dh[0]), 1.0 / (g.dh[1] * g.dh[1]), 1.0 / (g.dh[2] * g.dh[2])};
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    double acc = 0;
    for (int64_t u = (int64_t)blockIdx.x * AD_THREADS + threadIdx.x; u < nn; u += (int64_t)AD_BLOCKS * AD_THREADS) {
        const int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / sz);
        const bool interior = i > 0 && j > 0 && k > 0 && i < g.ni - 1 && j < g.nj - 1 && k < g.nk - 1;
        if (!interior || obj[u] != 0) {
            gn[u] = 0;
            continue;
        }
        const double l = lam[u];
        gn[u] = q * l / (AD_EPS_0 * vol[u]);
        const int64_t nb[6] = {u - 1, u + 1, u - sy, u + sy, u - sz, u + sz};
        double cs = 0;
        for (int m = 0; m < 6; m++)
            if (obj[nb[m]] == 1) cs += cd[m >> 1];
        acc += l * cs;
    }
    ad_block_store(acc, partials);
}

}  // namespace espic

/* ======================================================================== */
using namespace espic;

struct espic_world {
    World w;
};

struct espic_diff {
    World *w = nullptr;
    int prec = 0; /* 0: float64 particles and adjoints, 1: float32 */
    int64_t n = 0;
    int K = 20;
    double mass = 0, charge = 0, w0 = 0, alpha = 1, beta = 1;
    DiffGeo G{};
    size_t esz = 8;
    void *init = nullptr;      /* initial x, v (rows 0..5), w row filled by forward */
    void *cur = nullptr;       /* running state */
    void *seg = nullptr;       /* (K + 1) states of the segment being replayed */
    double *seg_phi = nullptr; /* (K + 1) potentials */
    std::vector<void *> ck_state;
    std::vector<double *> ck_phi;
    void *adj = nullptr; /* particle adjoints, rows as the state */
    double *Ebar = nullptr, *phib = nullptr, *lam = nullptr, *gn = nullptr;
    uint8_t *box = nullptr;
    double *d_part = nullptr, *d_acc = nullptr; /* [0] loss, [1] phi_s bar, [2] scratch */
    int nsteps = -1;
    double phi_s = 0;
};

static int dfail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return espic_internal_fail(code, buf);
}

#define DCK(call)                                                                                      \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess) return dfail(ESPIC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
    } while (0)

static void diff_free(espic_diff *d) {
    void *ptrs[] = {d->init, d->cur, d->seg, d->seg_phi, d->adj, d->Ebar, d->phib, d->lam, d->gn, d->box,
                    d->d_part, d->d_acc};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    for (void *p : d->ck_state) cudaFree(p);
    for (double *p : d->ck_phi) cudaFree(p);
    delete d;
}

static inline void *row_ptr(const espic_diff &D, void *base, int64_t k) {
    return (char *)base + (size_t)k * 7 * D.n * D.esz;
}

/* the Neumann chain targets the solve and the adjoint fold read */
static void diff_targets(World &w) {
    if (!w.targets_valid) {
        launch_targets(w);
        w.targets_valid = true;
    }
}

/* deposit of state P into w.rho and the Boltzmann solve into w.phi */
static int diff_field(espic_diff &D, const void *P) {
    World &w = *D.w;
    diff_targets(w);
    DCK(cudaMemsetAsync(w.rho, 0, w.nn * sizeof(double), w.stream));
    const int nb = blocks_for(D.n, 256);
    if (D.prec == 0)
        k_ad_deposit<double><<<nb, 256, 0, w.stream>>>(D.G, (const double *)P, D.n, D.charge, w.rho);
    else
        k_ad_deposit<float><<<nb, 256, 0, w.stream>>>(D.G, (const float *)P, D.n, D.charge, w.rho);
    k_ad_per_volume<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, w.rho, w.vol);
    k_ad_set_sphere<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, w.obj, D.phi_s, w.phi);
    w.nlaunch += 3;
    DCK(cudaGetLastError());
    int rc = launch_newton_pcg(w, D.prec == 1);
    if (rc) return dfail(ESPIC_ERR_CUDA, "Newton-PCG launch: %s", cudaGetErrorString((cudaError_t)rc));
    w.nlaunch++;
    return ESPIC_OK;
}

static int diff_push(espic_diff &D, const void *in, void *out) {
    World &w = *D.w;
    launch_efield(w);
    const int nb = blocks_for(D.n, 256);
    const double ke = D.charge / D.mass * w.dt;
    if (D.prec == 0)
        k_ad_push<double><<<nb, 256, 0, w.stream>>>(D.G, w.ef, (const double *)in, (double *)out, D.n, ke, w.dt);
    else
        k_ad_push<float><<<nb, 256, 0, w.stream>>>(D.G, w.ef, (const float *)in, (float *)out, D.n, (float)ke,
                                                   (float)w.dt);
    w.nlaunch++;
    DCK(cudaGetLastError());
    return ESPIC_OK;
}

static int diff_solve_adjoint(espic_diff &D, const void *P) {
    /* phi_bar in D.phib (all nodes), phi^n in w.phi: fold Neumann copies, the
     * direct sphere term, lambda = J^-1 phi_bar, then g and the sphere
     * coupling; then the deposit adjoint at P */
    World &w = *D.w;
    const int nbn = blocks_for(w.nn, 256);
    diff_targets(w);
    k_ad_fold<<<nbn, 256, 0, w.stream>>>(w.nn, w.target, D.phib);
    k_ad_sphere_direct<<<AD_BLOCKS, AD_THREADS, 0, w.stream>>>(w.nn, w.obj, D.phib, D.d_part);
    k_ad_final<<<1, 32, 0, w.stream>>>(D.d_part, 1.0, D.d_acc + 1, 1);
    DCK(cudaMemsetAsync(D.lam, 0, w.nn * sizeof(double), w.stream));
    w.nlaunch += 3;
    int rc = launch_pcg_linear(w, D.prec == 1, D.phib, D.lam, 1e-10, 10);
    if (rc) return dfail(ESPIC_ERR_CUDA, "adjoint PCG launch: %s", cudaGetErrorString((cudaError_t)rc));
    k_ad_after_solve<<<AD_BLOCKS, AD_THREADS, 0, w.stream>>>(w.g, w.obj, D.lam, w.vol, D.charge, D.gn, D.d_part);
    k_ad_final<<<1, 32, 0, w.stream>>>(D.d_part, 1.0, D.d_acc + 1, 1);
    const int nb = blocks_for(D.n, 256);
    if (D.prec == 0)
        k_ad_deposit_adj<double><<<nb, 256, 0, w.stream>>>(D.G, (const double *)P, D.n, D.gn, (double *)D.adj);
    else
        k_ad_deposit_adj<float><<<nb, 256, 0, w.stream>>>(D.G, (const float *)P, D.n, D.gn, (float *)D.adj);
    w.nlaunch += 4;
    DCK(cudaGetLastError());
    return ESPIC_OK;
}

extern "C" int espic_diff_create(espic_world *h, int precision, double mass, double charge, double mpw0, int64_t n,
                                 double delta, double wake_z0, double wake_z1, double alpha, double beta,
                                 int checkpoint_every, espic_diff **out) {
    if (!h || !out) return dfail(ESPIC_ERR_ARG, "null argument");
    *out = nullptr;
    World &w = h->w;
    if (cudaSetDevice(w.device) != cudaSuccess) return dfail(ESPIC_ERR_CUDA, "cudaSetDevice failed");
    if (precision != 0 && precision != 1) return dfail(ESPIC_ERR_ARG, "precision must be 0 (FP64) or 1 (FP32)");
    if (n < 1 || n > 0x7fffffffLL || !(mass > 0) || !(delta > 0) || checkpoint_every < 1)
        return dfail(ESPIC_ERR_ARG, "bad differentiable-run parameters");
    espic_diff *d = new espic_diff();
    espic_diff &D = *d;
    D.w = &w;
    D.prec = precision;
    D.esz = precision == 0 ? 8 : 4;
    D.n = n;
    D.K = checkpoint_every;
    D.mass = mass;
    D.charge = charge;
    D.w0 = mpw0;
    D.alpha = alpha;
    D.beta = beta;
    D.G.ni = w.g.ni;
    D.G.nj = w.g.nj;
    D.G.nk = w.g.nk;
    for (int k = 0; k < 3; k++) {
        D.G.x0[k] = w.g.x0[k];
        D.G.inv_dh[k] = 1.0 / w.g.dh[k];
        D.G.xmin[k] = w.g.x0[k];
        D.G.xmax[k] = w.g.xm[k];
        D.G.c[k] = w.sphere[k];
    }
    D.G.R = w.has_sphere ? sqrt(w.sphere[3]) : -1.0;
    D.G.delta = delta;
    const size_t st = (size_t)7 * n * D.esz;
    cudaError_t ce = cudaMalloc(&D.init, st);
    if (ce == cudaSuccess) ce = cudaMalloc(&D.cur, st);
    if (ce == cudaSuccess) ce = cudaMalloc(&D.seg, st * (D.K + 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.seg_phi, (size_t)w.nn * sizeof(double) * (D.K + 1));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.adj, st);
    if (ce == cudaSuccess) ce = cudaMalloc(&D.Ebar, (size_t)w.nn * 3 * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.phib, (size_t)w.nn * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.lam, (size_t)w.nn * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.gn, (size_t)w.nn * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.box, (size_t)w.nn);
    if (ce == cudaSuccess) ce = cudaMalloc(&D.d_part, AD_BLOCKS * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMalloc(&D.d_acc, 4 * sizeof(double));
    if (ce == cudaSuccess) ce = cudaMemset(D.init, 0, st);
    if (ce != cudaSuccess) {
        diff_free(d);
        return dfail(ESPIC_ERR_CUDA, "allocation: %s", cudaGetErrorString(ce));
    }
    /* wake-box node mask: nodes with z in [z0, z1] */
    std::vector<uint8_t> m((size_t)w.nn);
    for (int64_t u = 0; u < w.nn; u++) {
        int k = (int)(u / ((int64_t)w.g.ni * w.g.nj));
        double z = w.g.x0[2] + k * w.g.dh[2];
        m[u] = (z >= wake_z0 && z <= wake_z1) ? 1 : 0;
    }
    cudaMemcpy(D.box, m.data(), m.size(), cudaMemcpyHostToDevice);
    *out = d;
    return ESPIC_OK;
}

extern "C" void espic_diff_destroy(espic_diff *d) {
    if (!d) return;
    cudaSetDevice(d->w->device);
    cudaStreamSynchronize(d->w->stream);
    diff_free(d);
}

/* initial positions x[3][n] and velocities v[3][n] (float64) */
extern "C" int espic_diff_set_state(espic_diff *d, const double *x, const double *v) {
    if (!d || !x || !v) return dfail(ESPIC_ERR_ARG, "null argument");
    espic_diff &D = *d;
    World &w = *D.w;
    std::vector<double> buf((size_t)6 * D.n);
    std::copy(x, x + 3 * D.n, buf.begin());
    std::copy(v, v + 3 * D.n, buf.begin() + 3 * D.n);
    if (D.prec == 0) {
        DCK(cudaMemcpyAsync(D.init, buf.data(), buf.size() * 8, cudaMemcpyHostToDevice, w.stream));
    } else {
        std::vector<float> fb(buf.begin(), buf.end());
        DCK(cudaMemcpyAsync(D.init, fb.data(), fb.size() * 4, cudaMemcpyHostToDevice, w.stream));
    }
    DCK(cudaStreamSynchronize(w.stream));
    D.nsteps = -1;
    return ESPIC_OK;
}

/* the forward run of nsteps steps with the sphere at phi_s; stores
 * checkpoints and returns the loss */
extern "C" int espic_diff_forward(espic_diff *d, double phi_s, int nsteps, double *loss) {
    if (!d) return dfail(ESPIC_ERR_ARG, "null handle");
    espic_diff &D = *d;
    World &w = *D.w;
    if (nsteps < 0) return dfail(ESPIC_ERR_ARG, "nsteps must be >= 0");
    if (!(w.dt > 0)) return dfail(ESPIC_ERR_STATE, "setTime first");
    DCK(cudaSetDevice(w.device));
    D.phi_s = phi_s;
    const size_t st = (size_t)7 * D.n * D.esz;
    int nck = nsteps / D.K + 1;
    while ((int)D.ck_state.size() < nck) {
        void *a = nullptr;
        double *b = nullptr;
        DCK(cudaMalloc(&a, st));
        DCK(cudaMalloc(&b, (size_t)w.nn * sizeof(double)));
        D.ck_state.push_back(a);
        D.ck_phi.push_back(b);
    }
    DCK(cudaMemcpyAsync(D.cur, D.init, st, cudaMemcpyDeviceToDevice, w.stream));
    const int nb = blocks_for(D.n, 256);
    if (D.prec == 0)
        k_ad_weights0<double><<<nb, 256, 0, w.stream>>>(D.G, (double *)D.cur, D.n, D.w0);
    else
        k_ad_weights0<float><<<nb, 256, 0, w.stream>>>(D.G, (float *)D.cur, D.n, (float)D.w0);
    w.nlaunch++;
    DCK(cudaMemsetAsync(w.phi, 0, w.nn * sizeof(double), w.stream));
    int rc = diff_field(D, D.cur);
    if (rc) return rc;
    for (int s = 0; s < nsteps; s++) {
        if (s % D.K == 0) {
            DCK(cudaMemcpyAsync(D.ck_state[s / D.K], D.cur, st, cudaMemcpyDeviceToDevice, w.stream));
            DCK(cudaMemcpyAsync(D.ck_phi[s / D.K], w.phi, w.nn * sizeof(double), cudaMemcpyDeviceToDevice,
                                w.stream));
        }
        rc = diff_push(D, D.cur, D.cur);
        if (rc) return rc;
        rc = diff_field(D, D.cur);
        if (rc) return rc;
    }
    /* loss = alpha PE(phi^N) + beta wake ions */
    launch_efield(w);
    launch_pe(w, D.d_acc + 2);
    if (D.prec == 0)
        k_ad_wake<double><<<AD_BLOCKS, AD_THREADS, 0, w.stream>>>(D.G, (const double *)D.cur, D.n, D.box, D.d_part);
    else
        k_ad_wake<float><<<AD_BLOCKS, AD_THREADS, 0, w.stream>>>(D.G, (const float *)D.cur, D.n, D.box, D.d_part);
    k_ad_final<<<1, 32, 0, w.stream>>>(D.d_part, 1.0, D.d_acc + 3, 0);
    w.nlaunch += 2;
    DCK(cudaGetLastError());
    double h[2];
    DCK(cudaMemcpyAsync(h, D.d_acc + 2, 2 * sizeof(double), cudaMemcpyDeviceToHost, w.stream));
    DCK(cudaStreamSynchronize(w.stream));
    int bits = 0;
    DCK(cudaMemcpy(&bits, w.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (bits) {
        cudaMemset(w.d_err, 0, sizeof(int));
        return dfail(ESPIC_ERR_NONFINITE, "non-finite value in the differentiable forward");
    }
    D.nsteps = nsteps;
    if (loss) *loss = D.alpha * h[0] + D.beta * h[1];
    return ESPIC_OK;
}

/* gradients of the last forward's loss: d/d phi_s, d/d x^0 [3][n], d/d v^0
 * [3][n] (float64 on the host) */
extern "C" int espic_diff_backward(espic_diff *d, double *dphi_s, double *dx, double *dv) {
    if (!d) return dfail(ESPIC_ERR_ARG, "null handle");
    espic_diff &D = *d;
    World &w = *D.w;
    if (D.nsteps < 0) return dfail(ESPIC_ERR_STATE, "run espic_diff_forward first");
    DCK(cudaSetDevice(w.device));
    const int N = D.nsteps;
    const size_t st = (size_t)7 * D.n * D.esz;
    const int nb = blocks_for(D.n, 256), nbn = blocks_for(w.nn, 256);
    const double ke = D.charge / D.mass * w.dt;
    DCK(cudaMemsetAsync(D.d_acc + 1, 0, sizeof(double), w.stream));
    /* terminal: the state N is D.cur, phi^N in w.phi */
    if (D.prec == 0)
        k_ad_terminal<double><<<nb, 256, 0, w.stream>>>(D.G, (const double *)D.cur, D.n, D.box, D.beta,
                                                        (double *)D.adj);
    else
        k_ad_terminal<float><<<nb, 256, 0, w.stream>>>(D.G, (const float *)D.cur, D.n, D.box, (float)D.beta,
                                                       (float *)D.adj);
    launch_efield(w);
    k_ad_pe_adj<<<nbn, 256, 0, w.stream>>>(w.nn, w.ef, w.vol, D.alpha, D.Ebar);
    k_ad_gradT<<<nbn, 256, 0, w.stream>>>(w.g, D.Ebar, D.phib);
    w.nlaunch += 3;
    /* the final state for the deposit adjoint at N */
    void *PN = row_ptr(D, D.seg, 0);
    DCK(cudaMemcpyAsync(PN, D.cur, st, cudaMemcpyDeviceToDevice, w.stream));
    int rc = diff_solve_adjoint(D, PN);
    if (rc) return rc;
    /* segments, last first */
    for (int n1 = N; n1 > 0;) {
        const int n0 = ((n1 - 1) / D.K) * D.K;
        const int len = n1 - n0;
        /* replay n0 .. n1 from the checkpoint */
        DCK(cudaMemcpyAsync(row_ptr(D, D.seg, 0), D.ck_state[n0 / D.K], st, cudaMemcpyDeviceToDevice, w.stream));
        DCK(cudaMemcpyAsync(D.seg_phi, D.ck_phi[n0 / D.K], w.nn * sizeof(double), cudaMemcpyDeviceToDevice,
                            w.stream));
        DCK(cudaMemcpyAsync(w.phi, D.ck_phi[n0 / D.K], w.nn * sizeof(double), cudaMemcpyDeviceToDevice,
                            w.stream));
        for (int s = 0; s < len; s++) {
            rc = diff_push(D, row_ptr(D, D.seg, s), row_ptr(D, D.seg, s + 1));
            if (rc) return rc;
            if (s + 1 < len) {
                rc = diff_field(D, row_ptr(D, D.seg, s + 1));
                if (rc) return rc;
                DCK(cudaMemcpyAsync(D.seg_phi + (size_t)(s + 1) * w.nn, w.phi, w.nn * sizeof(double),
                                    cudaMemcpyDeviceToDevice, w.stream));
            }
        }
        /* adjoint steps n1-1 .. n0 */
        for (int s = len - 1; s >= 0; s--) {
            DCK(cudaMemcpyAsync(w.phi, D.seg_phi + (size_t)s * w.nn, w.nn * sizeof(double),
                                cudaMemcpyDeviceToDevice, w.stream));
            launch_efield(w);
            DCK(cudaMemsetAsync(D.Ebar, 0, (size_t)w.nn * 3 * sizeof(double), w.stream));
            if (D.prec == 0)
                k_ad_step<double><<<nb, 256, 0, w.stream>>>(D.G, w.ef, (const double *)row_ptr(D, D.seg, s),
                                                            (const double *)row_ptr(D, D.seg, s + 1), D.n, ke,
                                                            w.dt, (double *)D.adj, D.Ebar);
            else
                k_ad_step<float><<<nb, 256, 0, w.stream>>>(D.G, w.ef, (const float *)row_ptr(D, D.seg, s),
                                                           (const float *)row_ptr(D, D.seg, s + 1), D.n, (float)ke,
                                                           (float)w.dt, (float *)D.adj, D.Ebar);
            k_ad_gradT<<<nbn, 256, 0, w.stream>>>(w.g, D.Ebar, D.phib);
            w.nlaunch += 2;
            rc = diff_solve_adjoint(D, row_ptr(D, D.seg, s));
            if (rc) return rc;
        }
        n1 = n0;
    }
    /* the initial weights w0 a(x^0) */
    if (D.prec == 0)
        k_ad_initial<double><<<nb, 256, 0, w.stream>>>(D.G, (const double *)D.init, D.n, D.w0, (double *)D.adj);
    else
        k_ad_initial<float><<<nb, 256, 0, w.stream>>>(D.G, (const float *)D.init, D.n, (float)D.w0,
                                                      (float *)D.adj);
    w.nlaunch++;
    DCK(cudaGetLastError());
    double ps = 0;
    DCK(cudaMemcpyAsync(&ps, D.d_acc + 1, sizeof(double), cudaMemcpyDeviceToHost, w.stream));
    std::vector<double> A((size_t)6 * D.n);
    if (D.prec == 0) {
        DCK(cudaMemcpyAsync(A.data(), D.adj, A.size() * 8, cudaMemcpyDeviceToHost, w.stream));
        DCK(cudaStreamSynchronize(w.stream));
    } else {
        std::vector<float> f(A.size());
        DCK(cudaMemcpyAsync(f.data(), D.adj, f.size() * 4, cudaMemcpyDeviceToHost, w.stream));
        DCK(cudaStreamSynchronize(w.stream));
        std::copy(f.begin(), f.end(), A.begin());
    }
    if (dphi_s) *dphi_s = ps;
    if (dx) std::copy(A.begin(), A.begin() + 3 * D.n, dx);
    if (dv) std::copy(A.begin() + 3 * D.n, A.end(), dv);
    int bits = 0;
    DCK(cudaMemcpy(&bits, w.d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (bits) {
        cudaMemset(w.d_err, 0, sizeof(int));
        return dfail(ESPIC_ERR_NONFINITE, "non-finite value in the adjoint");
    }
    return ESPIC_OK;
}
