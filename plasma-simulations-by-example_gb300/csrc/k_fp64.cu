/*
 * k_fp64.cu -- the float64 plain form of the ES-PIC step, plus the field
 * kernels shared by both forms.  Compiled with -fmad=false: every product
 * and sum is rounded separately, in the reference's operand order, so that
 * positions, velocities, cell indices, absorbed counts and fields reproduce
 * the reference's g++ results bit for bit.
 *
 * Reference correspondence (file:line in the reference tree):
 *   gather           ch2/Field.h:186-208        k_push_fp64, gather3
 *   scatter          ch2/Field.h:164-183        deposit8 (fixed point)
 *   advance (box)    ch2/Species.cpp:7-38       k_push_fp64<REFLECT>
 *   advance (sphere) ch3/ver2/Species.cpp:7-48  k_push_fp64<ABSORB> + compaction
 *   addParticle      ch2/Species.cpp:55-71      k_append (all generators)
 *   computeEF        ch2/PotentialSolver.cpp:70-110   k_efield
 *   solve (SOR)      ch2/PotentialSolver.cpp:11-67    k_sor_box (red-black)
 *   solveGS          ch3/ver2/PotentialSolver.cpp:334-430 k_gs_sphere (red-black)
 *   solveQN          ch3/ver2/PotentialSolver.cpp:204-222 k_qn
 */
#include <cooperative_groups.h>
#include <limits.h>
#include <stdio.h>

#include <type_traits>

#include "ch4_push.h"
#include "dfloat.h"
#include "espic_world.h"

namespace cg = cooperative_groups;

namespace espic {

#define EPS_0 8.85418782e-12
#define QE 1.602176565e-19
#define KB 1.380648e-23
#define REF_PI 3.141592653

enum { REFLECT = 0, ABSORB = 1 };

__device__ __forceinline__ int clamp_cell(int i, int n) { return i < 0 ? 0 : (i > n - 2 ? n - 2 : i); }

__device__ __forceinline__ int64_t node_of(const Geo &g, int i, int j, int k) {
    return ((int64_t)k * g.nj + j) * g.ni + i;
}

/* Field_<double3>::gather with the index clamp: out-of-range truncated
 * indices (only reachable at x == xm after a one-bounce reflection) are
 * moved to n-2 keeping di = lc - i, which gives the same weights without
 * reading node n. */
__device__ __forceinline__ void gather3(const Geo &g, const double *__restrict__ ef, const double lc[3],
                                        double e[3]) {
    int i = clamp_cell((int)lc[0], g.ni), j = clamp_cell((int)lc[1], g.nj), k = clamp_cell((int)lc[2], g.nk);
    double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
    int64_t n0 = node_of(g, i, j, k);
    int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    const double *a = ef + 3 * n0;
    const double *b = ef + 3 * (n0 + 1);
    const double *c = ef + 3 * (n0 + 1 + sy);
    const double *d = ef + 3 * (n0 + sy);
    const double *e4 = ef + 3 * (n0 + sz);
    const double *f = ef + 3 * (n0 + 1 + sz);
    const double *h = ef + 3 * (n0 + 1 + sy + sz);
    const double *m = ef + 3 * (n0 + sy + sz);
#pragma unroll
    for (int q = 0; q < 3; q++) {
        e[q] = a[q] * (1 - di) * (1 - dj) * (1 - dk) + b[q] * (di) * (1 - dj) * (1 - dk) +
               c[q] * (di) * (dj) * (1 - dk) + d[q] * (1 - di) * (dj) * (1 - dk) +
               e4[q] * (1 - di) * (1 - dj) * (dk) + f[q] * (di) * (1 - dj) * (dk) +
               h[q] * (di) * (dj) * (dk) + m[q] * (1 - di) * (dj) * (dk);
    }
}

__device__ __forceinline__ void xtol(const Geo &g, const double x[3], double lc[3]) {
#pragma unroll
    for (int d = 0; d < 3; d++) lc[d] = (x[d] - g.x0[d]) / g.dh[d];
}

__device__ __forceinline__ bool in_bounds(const Geo &g, const double x[3]) {
#pragma unroll
    for (int d = 0; d < 3; d++)
        if (x[d] < g.x0[d] || x[d] >= g.xm[d]) return false;
    return true;
}

/* a / b correctly rounded, given y = RN(1/b) for b > 0: q = a y, the exact
 * remainder r = a - b q (one FMA), then q + r y rounded -- Markstein's
 * correction (P. Markstein, IBM J. Res. Develop. 34(1), 1990), which yields
 * the correctly rounded quotient for normal operands, so results equal the
 * division's bit for bit; a = +-0 returns a y, the zero of the right sign.
 * Three float64 operations instead of a division: the GB300's float64 rate
 * makes the division dominate the kernels below. */
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
    const double q = a * y;
    const double r = __fma_rn(-q, b, a);
    const double q2 = __fma_rn(r, y, q);
    /* a == +-0 tested on the bits: an integer compare keeps the narrow
     * float64 pipe for the arithmetic */
    return zero_bits(a) ? q : q2;
}

/* x to logical coordinates with the correctly rounded reciprocal of dh:
 * equal to World::XtoL's division bit for bit (div_rcp) */
__device__ __forceinline__ void xtol_rcp(const Geo &g, double3 rdh, const double x[3], double lc[3]) {
    lc[0] = div_rcp(x[0] - g.x0[0], g.dh[0], rdh.x);
    lc[1] = div_rcp(x[1] - g.x0[1], g.dh[1], rdh.y);
    lc[2] = div_rcp(x[2] - g.x0[2], g.dh[2], rdh.z);
}

__device__ __forceinline__ bool in_sphere(const double s[4], const double x[3]) {
    double r0 = x[0] - s[0], r1 = x[1] - s[1], r2 = x[2] - s[2];
    double rm2 = r0 * r0 + r1 * r1 + r2 * r2;
    return rm2 <= s[3];
}

/* Field_::scatter of `value` at x as 64-bit fixed point: each corner weight
 * value*(1-di)*(1-dj)*(1-dk) (reference order) is rounded once to an integer
 * count of 1/fx and added exactly. */
__device__ __forceinline__ void deposit8(const Geo &g, unsigned long long *acc, const double x[3],
                                         double value, double fx) {
    double lc[3];
    xtol(g, x, lc);
    int i = clamp_cell((int)lc[0], g.ni), j = clamp_cell((int)lc[1], g.nj), k = clamp_cell((int)lc[2], g.nk);
    double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
    int64_t n0 = node_of(g, i, j, k);
    int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    double w[8];
    w[0] = value * (1 - di) * (1 - dj) * (1 - dk);
    w[1] = value * (di) * (1 - dj) * (1 - dk);
    w[2] = value * (di) * (dj) * (1 - dk);
    w[3] = value * (1 - di) * (dj) * (1 - dk);
    w[4] = value * (1 - di) * (1 - dj) * (dk);
    w[5] = value * (di) * (1 - dj) * (dk);
    w[6] = value * (di) * (dj) * (dk);
    w[7] = value * (1 - di) * (dj) * (dk);
    int64_t idx[8] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy, n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
#pragma unroll
    for (int m = 0; m < 8; m++) {
        long long q = __double2ll_rn(w[m] * fx);
        if (q != 0) atomicAdd(acc + idx[m], (unsigned long long)q);
    }
}

/* ------------------------------------------------------------------------ */
/* Species::advance, fused with Species::computeNumberDensity of the moved
 * particles.  One thread per particle; a warp writes one word of the dead
 * mask and adds its dead count to the particle tile's counter. */
template <int WALLS, bool DEPOSIT, bool UNIFORM>
__global__ void __launch_bounds__(256) k_push_fp64(Geo g, const double *__restrict__ ef, double s,
                                                   double dt, double *P, int64_t stride,
                                                   const int64_t *__restrict__ d_count, double4 sph,
                                                   uint32_t *deadmask, int32_t *tiledead,
                                                   unsigned long long *acc, double fx, double w0,
                                                   int *err) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t n = d_count[0];
    bool dead = false;
    if (p < n) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        double lc[3], e[3];
        xtol(g, x, lc);
        gather3(g, ef, lc, e);
#pragma unroll
        for (int d = 0; d < 3; d++) v[d] += e[d] * s;
#pragma unroll
        for (int d = 0; d < 3; d++) x[d] += v[d] * dt;
        if (WALLS == REFLECT) {
#pragma unroll
            for (int d = 0; d < 3; d++) {
                if (x[d] < g.x0[d]) {
                    x[d] = 2 * g.x0[d] - x[d];
                    v[d] *= -1.0;
                } else if (x[d] >= g.xm[d]) {
                    x[d] = 2 * g.xm[d] - x[d];
                    v[d] *= -1.0;
                }
            }
        } else {
            double sp[4] = {sph.x, sph.y, sph.z, sph.w};
            dead = in_sphere(sp, x) || !in_bounds(g, x);
        }
        if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) {
            atomicOr(err, DERR_NONFINITE);
            dead = true;
        }
#pragma unroll
        for (int d = 0; d < 3; d++) {
            P[d * stride + p] = x[d];
            P[(3 + d) * stride + p] = v[d];
        }
        if (DEPOSIT && !dead) {
            double w = UNIFORM ? w0 : P[6 * stride + p];
            deposit8(g, acc, x, w, fx);
        }
    }
    if (WALLS == ABSORB) {
        unsigned m = __ballot_sync(0xffffffffu, dead);
        if ((threadIdx.x & 31) == 0 && p < n) {
            deadmask[p >> 5] = m;
            if (m) atomicAdd(tiledead + (p / TILE_PARTICLES), __popc(m));
        }
    }
}

template <bool UNIFORM>
__global__ void __launch_bounds__(256) k_deposit_fp64(Geo g, const double *__restrict__ P, int64_t stride,
                                                      const int64_t *__restrict__ d_count,
                                                      unsigned long long *acc, double fx, double w0) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d_count[0]) return;
    double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
    double w = UNIFORM ? w0 : P[6 * stride + p];
    deposit8(g, acc, x, w, fx);
}

/* ------------------------------------------------------------------------ */
/* Deterministic in-place compaction (both forms).  With D dead among n, the
 * r-th dead slot below n-D receives the r-th live particle at or above n-D.
 * 1) tile scan: exclusive prefix of dead counts per 32768-particle tile;
 * 2) holes: dead slots below n-D are listed by rank;
 * 3) movers: live particles at or above n-D copy into the hole of their rank. */
__global__ void __launch_bounds__(1024) k_tile_scan(int64_t *d_count, int32_t *tiledead, int32_t *tilepre) {
    __shared__ int32_t warp_sums[32];
    int64_t n = d_count[0];
    int64_t ntiles = (n + TILE_PARTICLES - 1) / TILE_PARTICLES;
    int t = threadIdx.x;
    int64_t per = (ntiles + blockDim.x - 1) / blockDim.x;
    int64_t a = t * per, b = a + per;
    if (b > ntiles) b = ntiles;
    int32_t sum = 0;
    for (int64_t i = a; i < b; i++) sum += tiledead[i];
    /* block exclusive scan of sum */
    int lane = t & 31, wid = t >> 5;
    int32_t incl = sum;
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_sums[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int32_t ws = warp_sums[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        warp_sums[lane] = ws;
    }
    __syncthreads();
    int32_t run = (wid ? warp_sums[wid - 1] : 0) + incl - sum;
    for (int64_t i = a; i < b; i++) {
        tilepre[i] = run;
        run += tiledead[i];
        tiledead[i] = 0; /* ready for the next push */
    }
    __syncthreads();
    if (t == blockDim.x - 1) {
        int64_t D = run;
        tilepre[ntiles] = (int32_t)D;
        d_count[1] = n;     /* count before compaction */
        d_count[2] = D;     /* dead */
        d_count[0] = n - D; /* count after */
    }
}

/* block-wide exclusive scan helper for 1024 threads */
__device__ __forceinline__ int32_t block_excl_scan(int32_t v, int32_t *sh, int32_t *total) {
    int t = threadIdx.x, lane = t & 31, wid = t >> 5;
    int32_t incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        int32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) sh[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        int32_t ws = sh[lane];
        for (int o = 1; o < 32; o <<= 1) {
            int32_t y = __shfl_up_sync(0xffffffffu, ws, o);
            if (lane >= o) ws += y;
        }
        sh[lane] = ws;
    }
    __syncthreads();
    int32_t r = (wid ? sh[wid - 1] : 0) + incl - v;
    if (total) *total = sh[31];
    __syncthreads();
    return r;
}

/* one block per tile, one thread per 32-particle mask word */
__global__ void __launch_bounds__(1024) k_holes(const int64_t *__restrict__ d_count,
                                                const uint32_t *__restrict__ deadmask,
                                                const int32_t *__restrict__ tilepre, int32_t *holes) {
    __shared__ int32_t sh[32];
    int64_t n_old = d_count[1], n_new = d_count[0];
    int64_t ntiles = (n_old + TILE_PARTICLES - 1) / TILE_PARTICLES;
    for (int64_t T = blockIdx.x; T < ntiles; T += gridDim.x) {
        if (tilepre[T + 1] == tilepre[T]) continue;        /* no dead in tile */
        if ((int64_t)T * TILE_PARTICLES >= n_new) continue; /* tile entirely above n_new */
        int64_t word = T * (TILE_PARTICLES / 32) + threadIdx.x;
        uint32_t m = (word * 32 < n_old) ? deadmask[word] : 0u;
        int32_t pre = block_excl_scan(__popc(m), sh, nullptr);
        int32_t base = tilepre[T] + pre;
        while (m) {
            int b = __ffs(m) - 1;
            m &= m - 1;
            int64_t idx = word * 32 + b;
            if (idx < n_new) holes[base] = (int32_t)idx;
            base++;
        }
    }
}

/* number of dead particles with index < x (x <= n_old) */
__device__ int64_t dead_before(int64_t x, const uint32_t *deadmask, const int32_t *tilepre, int32_t *sh) {
    int64_t T = x / TILE_PARTICLES;
    int64_t w0 = T * (TILE_PARTICLES / 32);
    int64_t wx = x >> 5;
    int64_t word = w0 + threadIdx.x;
    int32_t c = 0;
    if (word < wx) c = __popc(deadmask[word]);
    else if (word == wx && (x & 31)) c = __popc(deadmask[word] & ((1u << (x & 31)) - 1u));
    int32_t tot;
    block_excl_scan(c, sh, &tot);
    return (int64_t)tilepre[T] + tot;
}

template <int FORM>
__device__ __forceinline__ void move_particle(int64_t dst, int64_t src, double *P, int32_t *cell, float *off,
                                              float *vel, int64_t stride, int rows) {
    if (FORM == 0) {
        for (int c = 0; c < rows; c++) P[c * stride + dst] = P[c * stride + src];
    } else {
        cell[dst] = cell[src];
#pragma unroll
        for (int c = 0; c < 3; c++) {
            off[c * stride + dst] = off[c * stride + src];
            vel[c * stride + dst] = vel[c * stride + src];
        }
    }
}

/* one block per 1024-particle chunk of the tail [n_new, n_old), one thread
 * per particle (warp w holds mask word w of the chunk) */
template <int FORM>
__global__ void __launch_bounds__(1024) k_movers(const int64_t *__restrict__ d_count,
                                                 const uint32_t *__restrict__ deadmask,
                                                 const int32_t *__restrict__ tilepre,
                                                 const int32_t *__restrict__ holes, double *P, int32_t *cell,
                                                 float *off, float *vel, int64_t stride, int rows) {
    __shared__ int32_t sh[32];
    __shared__ int32_t wsum[32];
    int64_t n_old = d_count[1], n_new = d_count[0];
    if (n_old == n_new) return;
    const int64_t c0 = n_new >> 10, c1 = (n_old - 1) >> 10;
    if (c0 + (int64_t)blockIdx.x > c1) return;
    const int64_t dead_at_new = dead_before(n_new, deadmask, tilepre, sh);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int64_t c = c0 + blockIdx.x; c <= c1; c += gridDim.x) {
        /* dead particles in the chunk's tile before the chunk */
        int64_t T = (c << 10) / TILE_PARTICLES;
        int64_t wt0 = T * (TILE_PARTICLES / 32), wc0 = c * 32;
        int64_t word_t = wt0 + threadIdx.x;
        int32_t cnt = (word_t < wc0) ? __popc(deadmask[word_t]) : 0;
        int32_t tot;
        block_excl_scan(cnt, sh, &tot);
        const int64_t dead_before_chunk = (int64_t)tilepre[T] + tot;
        /* the chunk's words */
        int64_t word = wc0 + warp;
        uint32_t m = (word * 32 < n_old) ? deadmask[word] : 0xffffffffu;
        if (lane == 0) wsum[warp] = __popc(m);
        __syncthreads();
        int32_t wpre = 0;
        for (int k = 0; k < warp; k++) wpre += wsum[k];
        int64_t q = word * 32 + lane;
        if (q >= n_new && q < n_old && !((m >> lane) & 1u)) {
            int64_t db = dead_before_chunk + wpre + __popc(m & ((1u << lane) - 1u));
            int64_t rank = (q - n_new) - (db - dead_at_new);
            move_particle<FORM>(holes[rank], q, P, cell, off, vel, stride, rows);
        }
        __syncthreads();
    }
}

/* ------------------------------------------------------------------------ */
/* Candidate generators for appended particles.  Each produces the position,
 * velocity and weight of candidate i exactly as the reference's loader or
 * source computes them before calling addParticle. */
struct GenHost { /* Species::addParticle from a host list */
    const double *pos3, *vel3, *w;
    double w0;
    __device__ void make(int64_t i, double x[3], double v[3], double &w_) const {
        for (int d = 0; d < 3; d++) {
            x[d] = pos3[3 * i + d];
            v[d] = vel3[3 * i + d];
        }
        w_ = w ? w[i] : w0;
    }
    __device__ void pos(int64_t i, double x[3]) const {
        for (int d = 0; d < 3; d++) x[d] = pos3[3 * i + d];
    }
};

struct GenBox { /* Species::loadParticlesBox, ch2/Species.cpp:74-97 */
    double x1[3], x2[3], mpw;
    const double *u; /* 3 per particle or null -> Philox */
    uint64_t seed, stream;
    __device__ double U(int64_t k) const { return u ? u[k] : philox_uniform(seed, stream, (uint64_t)k); }
    __device__ void pos(int64_t i, double x[3]) const {
        for (int d = 0; d < 3; d++) x[d] = x1[d] + U(3 * i + d) * (x2[d] - x1[d]);
    }
    __device__ void make(int64_t i, double x[3], double v[3], double &w_) const {
        pos(i, x);
        v[0] = v[1] = v[2] = 0;
        w_ = mpw;
    }
};

struct GenQS { /* Species::loadParticlesBoxQS, ch2/Species.cpp:101-141 */
    double x1[3], x2[3], mpw, di, dj, dk;
    int n0, n1, n2;
    __device__ void idx(int64_t t, int &i, int &j, int &k) const {
        k = (int)(t % n2);
        int64_t r = t / n2;
        j = (int)(r % n1);
        i = (int)(r / n1);
    }
    __device__ void pos(int64_t t, double x[3]) const {
        int i, j, k;
        idx(t, i, j, k);
        x[0] = x1[0] + i * di;
        x[1] = x1[1] + j * dj;
        x[2] = x1[2] + k * dk;
        if (x[0] == x2[0]) x[0] -= 1e-4 * di;
        if (x[1] == x2[1]) x[1] -= 1e-4 * dj;
        if (x[2] == x2[2]) x[2] -= 1e-4 * dk;
    }
    __device__ void make(int64_t t, double x[3], double v[3], double &w_) const {
        pos(t, x);
        int i, j, k;
        idx(t, i, j, k);
        double w = 1;
        if (i == 0 || i == n0 - 1) w *= 0.5;
        if (j == 0 || j == n1 - 1) w *= 0.5;
        if (k == 0 || k == n2 - 1) w *= 0.5;
        v[0] = v[1] = v[2] = 0;
        w_ = mpw * w;
    }
};

struct GenBeam { /* ColdBeamSource::sample (ch3/ver2/Source.cpp:4-27),
                    WarmBeamSource::sample (ch4/Source.cpp:31-55),
                    Source::sample of ch9/MPI (ch9/MPI/src/Source.cpp:5-72)
                    and a drifting-Maxwellian beam */
    double x0[3], Lx, Ly, v_drift, mpw0, v_th;
    double ncx, ncy, dhx, dhy; /* cells and spacing across the face (ch9/MPI's position formula) */
    int mode; /* 0 cold, 1 ch4 warm, 2 ch9 isotropic, 3 Maxwellian */
    const double *u; /* count draw at 0, then beam_uniforms(mode) per particle */
    uint64_t seed, stream;
    __device__ double U(int64_t k) const { return u ? u[k] : philox_uniform(seed, stream, (uint64_t)k); }
    __device__ int64_t base(int64_t i) const { return 1 + (int64_t)beam_uniforms(mode) * i; }
    __device__ void pos(int64_t i, double x[3]) const {
        int64_t b = base(i);
        if (mode == 2) { /* x0 + U (ni-1) dh, ch9/MPI/src/Source.cpp:33-35 */
            x[0] = x0[0] + U(b) * ncx * dhx;
            x[1] = x0[1] + U(b + 1) * ncy * dhy;
        } else {
            x[0] = x0[0] + U(b) * Lx;
            x[1] = x0[1] + U(b + 1) * Ly;
        }
        x[2] = x0[2];
    }
    __device__ void make(int64_t i, double x[3], double v[3], double &w_) const {
        pos(i, x);
        w_ = mpw0;
        if (mode == 0) {
            v[0] = 0;
            v[1] = 0;
            v[2] = v_drift;
            return;
        }
        if (mode == 2) {
            /* isotropic direction at speed v_th, drift added, v_z < 0
             * reflected (ch9/MPI/src/Source.cpp:39-59, PI = acos(-1)) */
            int64_t b = base(i) + 2;
            double theta = 2 * 3.141592653589793 * U(b);
            double r = -1.0 + 2 * U(b + 1);
            double a = sqrt(1 - r * r);
            v[0] = v_th * (cos(theta) * a);
            v[1] = v_th * (sin(theta) * a);
            v[2] = v_th * r + v_drift;
            if (v[2] < 0) v[2] = -v[2];
            return;
        }
        if (mode == 3) {
            /* drifting Maxwellian: normal components by Box-Muller with
             * sigma = v_th (here sqrt(kT/m)), v_z < 0 reflected as above */
            int64_t b = base(i) + 2;
            double r1 = sqrt(-2.0 * log(1.0 - U(b))), a1 = 2 * 3.141592653589793 * U(b + 1);
            double r2 = sqrt(-2.0 * log(1.0 - U(b + 2))), a2 = 2 * 3.141592653589793 * U(b + 3);
            v[0] = v_th * (r1 * cos(a1));
            v[1] = v_th * (r1 * sin(a1));
            v[2] = v_th * (r2 * cos(a2)) + v_drift;
            if (v[2] < 0) v[2] = -v[2];
            return;
        }
        /* Species::sampleIsotropicVel and sampleVth, ch4/Species.cpp:149-175 */
        int64_t b = base(i) + 2;
        double theta = 2 * REF_PI * U(b);
        double r = -1.0 + 2 * U(b + 1);
        double a = sqrt(1 - r * r);
        double d[3] = {r, cos(theta) * a, sin(theta) * a};
        double v1 = v_th * (U(b + 2) + U(b + 3) + U(b + 4) - 1.5);
        double v2 = v_th * (U(b + 5) + U(b + 6) + U(b + 7) - 1.5);
        double v3 = v_th * (U(b + 8) + U(b + 9) + U(b + 10) - 1.5);
        double speed = 3 / sqrt(6.0) * sqrt(v1 * v1 + v2 * v2 + v3 * v3);
        for (int c = 0; c < 3; c++) v[c] = d[c] * speed;
        v[2] += v_drift;
    }
};

struct GenThermal { /* uniform box with a drifting Maxwellian (no reference counterpart) */
    double x1[3], x2[3], mpw, sigma, vd[3];
    const double *u; /* 7 per particle or null -> Philox */
    uint64_t seed, stream;
    __device__ double U(int64_t k) const { return u ? u[k] : philox_uniform(seed, stream, (uint64_t)k); }
    __device__ void pos(int64_t i, double x[3]) const {
        for (int d = 0; d < 3; d++) x[d] = x1[d] + U(7 * i + d) * (x2[d] - x1[d]);
    }
    __device__ void make(int64_t i, double x[3], double v[3], double &w_) const {
        pos(i, x);
        /* Box-Muller: 1-u keeps the logarithm finite */
        double r1 = sqrt(-2.0 * log(1.0 - U(7 * i + 3))), a1 = 2 * REF_PI * U(7 * i + 4);
        double r2 = sqrt(-2.0 * log(1.0 - U(7 * i + 5))), a2 = 2 * REF_PI * U(7 * i + 6);
        v[0] = vd[0] + sigma * (r1 * cos(a1));
        v[1] = vd[1] + sigma * (r1 * sin(a1));
        v[2] = vd[2] + sigma * (r2 * cos(a2));
        w_ = mpw;
    }
};

/* Candidates per block of the append passes: small blocks spread an
 * injection of a few thousand candidates, whose float64 Box-Muller
 * transcendentals dominate, over many SMs. */
constexpr int APPEND_THREADS = 64;

/* Pass 1: accepted candidates per block (addParticle rejects x outside
 * [x0,xm)). */
template <class Gen>
__global__ void __launch_bounds__(APPEND_THREADS) k_append_count(Geo g, Gen gen, int64_t ncand, int32_t *blockcnt) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool ok = false;
    if (i < ncand) {
        double x[3];
        gen.pos(i, x);
        ok = in_bounds(g, x);
    }
    int c = __syncthreads_count(ok);
    if (threadIdx.x == 0) blockcnt[blockIdx.x] = c;
}

/* Pass 2 (one block): exclusive prefix of the block counts in place; the
 * particle count before the append goes to d_count[1], the new count (at
 * most the capacity) to d_count[0]. */
__global__ void __launch_bounds__(1024) k_append_scan(int32_t *blockcnt, int64_t nblocks, int64_t *d_count,
                                                      int64_t cap, int *err) {
    __shared__ int32_t sh[32];
    int t = threadIdx.x;
    int64_t per = (nblocks + blockDim.x - 1) / blockDim.x;
    int64_t a = t * per, b = a + per;
    if (b > nblocks) b = nblocks;
    int64_t sum = 0;
    for (int64_t i = a; i < b; i++) sum += blockcnt[i];
    int32_t total;
    int32_t run = block_excl_scan((int32_t)sum, sh, &total);
    for (int64_t i = a; i < b; i++) {
        int32_t c = blockcnt[i];
        blockcnt[i] = run;
        run += c;
    }
    if (t == 0) {
        int64_t n_old = d_count[0];
        int64_t n_new = n_old + total;
        if (n_new > cap) {
            atomicOr(err, DERR_CAPACITY);
            n_new = cap;
        }
        d_count[1] = n_old;
        d_count[0] = n_new;
    }
}

/* Pass 3: each accepted candidate is rewound by (q/m)E dt/2 and written at
 * n_old + (number of accepted candidates before it), so the order is the
 * candidates' order, as the reference's emplace_back.  The float64 form
 * gathers E from the float64 field in the reference's arithmetic; the mixed
 * form from the float copy ef4 with the mixed push's float weights (its
 * velocities are floats: the float64 gather cost ~100 float64 operations a
 * particle for a change below their last bit but one), with qmdt2 =
 * RN_f(q/m dt/2). */
template <class Gen, int FORM>
__global__ void __launch_bounds__(APPEND_THREADS) k_append_write(Geo g, double3 rdh, Gen gen, int64_t ncand,
                                                      const int32_t *__restrict__ blockpre,
                                                      const int64_t *__restrict__ d_count,
                                                      const double *__restrict__ ef, const float4 *__restrict__ ef4,
                                                      double qm, double dt, float qmdt2, double *P, int32_t *cell,
                                                      float *off, float *vel, int64_t stride, int64_t cap,
                                                      int write_w) {
    __shared__ int32_t sh[APPEND_THREADS / 32];
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t s_base = d_count[1] + blockpre[blockIdx.x];
    double x[3], v[3], w = 0;
    bool ok = false;
    if (i < ncand) {
        gen.make(i, x, v, w);
        ok = in_bounds(g, x);
    }
    /* block exclusive rank of ok */
    unsigned bal = __ballot_sync(0xffffffffu, ok);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = __popc(bal);
    __syncthreads();
    int32_t pre = 0;
    for (int k = 0; k < wid; k++) pre += sh[k];
    pre += __popc(bal & ((1u << lane) - 1u));
    if (ok) {
        int64_t dst = s_base + pre;
        if (dst < cap) {
            double lc[3];
            xtol_rcp(g, rdh, x, lc);
            if (FORM == 0) {
                double e[3];
                gather3(g, ef, lc, e);
                for (int d = 0; d < 3; d++) v[d] = v[d] - e[d] * qm * (0.5 * dt);
                for (int d = 0; d < 3; d++) {
                    P[d * stride + dst] = x[d];
                    P[(3 + d) * stride + dst] = v[d];
                }
                if (write_w) P[6 * stride + dst] = w;
            } else {
                int ci = clamp_cell((int)lc[0], g.ni), cj = clamp_cell((int)lc[1], g.nj),
                    ck = clamp_cell((int)lc[2], g.nk);
                const float fx = (float)(lc[0] - ci), fy = (float)(lc[1] - cj), fz = (float)(lc[2] - ck);
                float wc[8];
                cic_w(fx, fy, fz, wc);
                const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
                const float4 *E0 = ef4 + node_of(g, ci, cj, ck);
                const float4 e[8] = {__ldg(E0),      __ldg(E0 + 1),      __ldg(E0 + 1 + sy),      __ldg(E0 + sy),
                                     __ldg(E0 + sz), __ldg(E0 + 1 + sz), __ldg(E0 + 1 + sy + sz), __ldg(E0 + sy + sz)};
                const float3 E = gather_corners(wc, e);
                cell[dst] = ci | (cj << 10) | (ck << 20);
                off[dst] = fx;
                off[stride + dst] = fy;
                off[2 * stride + dst] = fz;
                vel[dst] = __fmaf_rn(-E.x, qmdt2, (float)v[0]);
                vel[stride + dst] = __fmaf_rn(-E.y, qmdt2, (float)v[1]);
                vel[2 * stride + dst] = __fmaf_rn(-E.z, qmdt2, (float)v[2]);
            }
        }
    }
}

/* ------------------------------------------------------------------------ */

/* PotentialSolver::computeEF: 2nd-order one-sided differences on the faces,
 * central inside.  Also writes the float32 copy used by the mixed push. */
/* The numerator of one component at node u with stride st along an axis of
 * n nodes at index i: one-sided on the faces, central inside, each in the
 * reference's arithmetic (ch2/PotentialSolver.cpp:70-110). */
__device__ __forceinline__ double ef_num(const double *__restrict__ phi, int64_t u, int64_t st, int i, int n) {
    if (i == 0) return -(-3 * phi[u] + 4 * phi[u + st] - phi[u + 2 * st]);
    if (i == n - 1) return -(phi[u - 2 * st] - 4 * phi[u - st] + 3 * phi[u]);
    return -(phi[u + st] - phi[u - st]);
}

/* grid: x over the nodes of a k-plane, y over the planes (no 64-bit index
 * division per node).  Interior nodes take the central differences alone:
 * the face formulas sit behind a branch the whole warp skips, so their
 * float64 operations are not issued for every node (this GPU's float64 rate
 * bounds the kernel). */
__global__ void __launch_bounds__(256) k_efield(Geo g, double3 y2, const double *__restrict__ phi, double *ef,
                                                float4 *ef4) {
    const uint32_t pl = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nplane = (uint32_t)g.ni * (uint32_t)g.nj;
    if (pl >= nplane) return;
    const int k = blockIdx.y;
    const uint32_t jj = div_small(pl, (uint32_t)g.ni, 1.f / (float)g.ni);
    const int j = (int)jj, i = (int)(pl - jj * (uint32_t)g.ni);
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    const int64_t u = (int64_t)k * sz + pl;
    const double d2x = 2 * g.dh[0], d2y = 2 * g.dh[1], d2z = 2 * g.dh[2];
    double n0, n1, n2;
    if (i > 0 && i < g.ni - 1 && j > 0 && j < g.nj - 1 && k > 0 && k < g.nk - 1) {
        n0 = -(phi[u + 1] - phi[u - 1]);
        n1 = -(phi[u + sy] - phi[u - sy]);
        n2 = -(phi[u + sz] - phi[u - sz]);
    } else {
        n0 = ef_num(phi, u, 1, i, g.ni);
        n1 = ef_num(phi, u, sy, j, g.nj);
        n2 = ef_num(phi, u, sz, k, g.nk);
    }
    const double e0 = div_rcp(n0, d2x, y2.x);
    const double e1 = div_rcp(n1, d2y, y2.y);
    const double e2 = div_rcp(n2, d2z, y2.z);
    ef[3 * u] = e0;
    ef[3 * u + 1] = e1;
    ef[3 * u + 2] = e2;
    if (ef4) ef4[u] = make_float4((float)e0, (float)e1, (float)e2, 0.f);
}

/* ------------------------------------------------------------------------ */
/* computeEF for worlds whose particles all live in the mixed form: the
 * float copy ef4 = RN_f(RN_d(n / 2dh)) of every node, bit for bit that of
 * k_efield.  Interior nodes take the float64 differences n (the reference's
 * numerators: three float64 operations) and the rest on the float and
 * integer pipes: q = n (-1 / 2dh) in double-float (within 2^-45 |q| of the
 * float64 quotient), rounded to float where it lies farther than 2^-40 |q|
 * from a float rounding boundary.  The faces, and the rare interior node
 * with a component near a boundary or outside the double-float range, take
 * ef_node_exact.  The float64 field is written on the planes k < 2 alone,
 * the ones a float64-form beam source's addParticle gathers at (its
 * particles start at z = x0; the mixed form's gathers from ef4); the rest
 * of it is completed on demand by k_efield from phi_ef,
 * the copy of phi this kernel reads (the solver changes phi before the
 * field is next computed, and the reference's ef stays that of the last
 * computeEF).  World::getPE's sum of |E|^2 vol over the nodes rides along
 * from the same q, in double-float (each term within 2^-44 of the float64
 * term, far inside the 1e-13 to which the sum's order already defines it).
 * Each thread takes EF_KPT planes of its (i, j) column, so the block sum is
 * paid once per EF_KPT nodes: one partial per block, [plane group][block of
 * the plane]. */
constexpr int EF_KPT = 8; /* planes per thread of k_efield4 */

struct EfConst {
    double3 y2, d2; /* RN(1 / 2dh) and 2 dh per axis */
    float2 ny[3];   /* -RN(1 / 2dh) as a float pair (hi, lo) */
};

/* one node of k_efield4 in float64: the numerators of ef_num, div_rcp, ef4
 * (and ef on the planes k < 2); returns pe + |E|^2 vol.  Not inlined, so
 * that it is a real branch: inlined, its float64 operations were
 * if-converted and issued for every node. */
__device__ __noinline__ double ef_node_exact(const double *__restrict__ phi, double *ef, float4 *ef4,
                                             const double *__restrict__ vol, int64_t u, int i, int j, int k, int ni,
                                             int nj, int nk, double3 d2, double3 y2, double pe) {
    const int64_t sy = ni, sz = (int64_t)ni * nj;
    const double e0 = div_rcp(ef_num(phi, u, 1, i, ni), d2.x, y2.x);
    const double e1 = div_rcp(ef_num(phi, u, sy, j, nj), d2.y, y2.y);
    const double e2 = div_rcp(ef_num(phi, u, sz, k, nk), d2.z, y2.z);
    if (k < 2) {
        ef[3 * u] = e0;
        ef[3 * u + 1] = e1;
        ef[3 * u + 2] = e2;
    }
    ef4[u] = make_float4((float)e0, (float)e1, (float)e2, 0.f);
    return __fma_rn(__fma_rn(e2, e2, __fma_rn(e1, e1, e0 * e0)), vol[u], pe);
}

__global__ void __launch_bounds__(256) k_efield4(Geo g, EfConst ec, const double *__restrict__ phi, double *ef,
                                                 float4 *ef4, const double *__restrict__ vol, double *pe_part,
                                                 double *phi_ef) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ni = (uint32_t)g.ni, nj = (uint32_t)g.nj, nplane = ni * nj;
    double pe = 0;         /* the nodes of ef_node_exact */
    dfl pe_d = {0.f, 0.f}; /* the rest, in double-float */
    if (t < nplane) {
        /* threads [0, (ni-2)(nj-2)) take the columns off the i and j faces,
         * i fastest; the rest take the face columns (the rows j = 0 and
         * j = nj-1, then the columns i = 0 and i = ni-1), so that a warp's
         * face nodes, which take ef_node_exact, share that call */
        const uint32_t nin = (ni > 2 && nj > 2) ? (ni - 2) * (nj - 2) : 0u;
        uint32_t i, j;
        if (t < nin) {
            const uint32_t jj = div_small(t, ni - 2, 1.f / (float)(ni - 2));
            j = 1 + jj;
            i = 1 + (t - jj * (ni - 2));
        } else {
            const uint32_t f = t - nin;
            if (f < 2 * ni) {
                j = f < ni ? 0u : nj - 1;
                i = f < ni ? f : f - ni;
            } else {
                const uint32_t f2 = f - 2 * ni;
                i = f2 < nj - 2 ? 0u : ni - 1;
                j = 1 + (f2 < nj - 2 ? f2 : f2 - (nj - 2));
            }
        }
        const uint32_t pl = j * ni + i;
        const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
        const bool in_ij = t < nin;
        const int k0 = blockIdx.y * EF_KPT;
        for (int kk = 0; kk < EF_KPT; kk++) {
            const int k = k0 + kk;
            if (k >= g.nk) break;
            const int64_t u = (int64_t)k * sz + pl;
            phi_ef[u] = phi[u];
            bool exact = !(in_ij && k >= 2 && k < g.nk - 1);
            if (!exact) {
                const double dd[3] = {phi[u + 1] - phi[u - 1], phi[u + sy] - phi[u - sy], phi[u + sz] - phi[u - sz]};
                float f[3];
                dfl e2 = {0.f, 0.f};
#pragma unroll
                for (int c = 0; c < 3; c++) {
                    dfl qd = {0.f, 0.f}, dv;
                    if (df_split_int(dd[c], dv)) {
                        qd = df_mul(dv, df_unpack(ec.ny[c]));
                        if (!f32_of_df(qd, 9.1e-13f * fabsf(qd.h), f[c])) exact = true;
                    } else {
                        if (zero_bits(dd[c])) /* -dd / 2dh: the zero of the opposite sign */
                            f[c] = __uint_as_float(((unsigned int)__double2hiint(dd[c]) & 0x80000000u) ^ 0x80000000u);
                        else
                            exact = true;
                    }
                    e2 = df_add(e2, df_mul(qd, qd));
                }
                dfl vd = {0.f, 0.f};
                if (!df_split_int(vol[u], vd)) exact = true;
                const dfl t = df_mul(e2, vd);
                /* terms of magnitude in [2^-100, 2^100] keep ~48 bits in
                 * double-float (a zero e2 is all three components zero) */
                const unsigned int te = __float_as_uint(t.h) & 0x7f800000u,
                                   ee = __float_as_uint(e2.h) & 0x7f800000u;
                if (!((te >= (27u << 23) && te <= (227u << 23) && ee >= (27u << 23) && ee <= (227u << 23)) ||
                      (__float_as_uint(e2.h) << 1) == 0u))
                    exact = true;
                if (!exact) {
                    ef4[u] = make_float4(f[0], f[1], f[2], 0.f);
                    pe_d = df_add(pe_d, t);
                }
            }
            if (exact) pe = ef_node_exact(phi, ef, ef4, vol, u, (int)i, (int)j, k, g.ni, g.nj, g.nk, ec.d2, ec.y2, pe);
        }
    }
    pe += (double)pe_d.h + (double)pe_d.l;
    /* deterministic block sum: warp butterflies, then the 8 warps in order */
    __shared__ double ws[8];
    for (int o = 16; o > 0; o >>= 1) pe += __shfl_xor_sync(0xffffffffu, pe, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = pe;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w8 = 0; w8 < (int)(blockDim.x >> 5); w8++) t += ws[w8];
        pe_part[(int64_t)blockIdx.y * gridDim.x + blockIdx.x] = t;
    }
}

/* ------------------------------------------------------------------------ */
/* World::addSphere: node position x0 + dh*(i,j,k), inside or on the sphere */
__global__ void k_objects_sphere(Geo g, double4 sph, double phi_s, int32_t *obj, double *phi) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    double l[3] = {(double)(u % g.ni), (double)((u / g.ni) % g.nj), (double)(u / ((int64_t)g.ni * g.nj))};
    double x[3];
    for (int d = 0; d < 3; d++) x[d] = g.x0[d] + g.dh[d] * l[d];
    double s[4] = {sph.x, sph.y, sph.z, sph.w};
    if (in_sphere(s, x)) {
        obj[u] = 1;
        phi[u] = phi_s;
    }
}

/* World::addInlet: the k = 0 plane is Dirichlet 0 V */
__global__ void k_objects_inlet(Geo g, int32_t *obj, double *phi) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= (int64_t)g.ni * g.nj) return;
    obj[u] = 2;
    phi[u] = 0;
}

/* immediate Neumann neighbour in the precedence of solveGS,
 * ch3/ver2/PotentialSolver.cpp:359-370; -1 for interior nodes */
__device__ __forceinline__ int64_t neumann_next(const Geo &g, int i, int j, int k) {
    if (i == 0) return node_of(g, i + 1, j, k);
    if (i == g.ni - 1) return node_of(g, i - 1, j, k);
    if (j == 0) return node_of(g, i, j + 1, k);
    if (j == g.nj - 1) return node_of(g, i, j - 1, k);
    if (k == 0) return node_of(g, i, j, k + 1);
    if (k == g.nk - 1) return node_of(g, i, j, k - 1);
    return -1;
}

/* end of each boundary node's chain of Neumann copies (-1 elsewhere) */
__global__ void k_targets(Geo g, const int32_t *__restrict__ obj, int32_t *target) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    target[u] = -1;
    if (obj[u] > 0) return;
    int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
    int64_t t = neumann_next(g, i, j, k);
    if (t < 0) return;
    for (int guard = 0; guard < 8; guard++) {
        if (obj[t] > 0) break;
        int ti = (int)(t % g.ni), tj = (int)((t / g.ni) % g.nj), tk = (int)(t / ((int64_t)g.ni * g.nj));
        int64_t n2 = neumann_next(g, ti, tj, tk);
        if (n2 < 0) break;
        t = n2;
    }
    target[u] = (int32_t)t;
}

/* ------------------------------------------------------------------------ */
/* den = acc * unit / node_vol (0 where the volume is 0): the fixed-point sum
 * followed by Field_::operator/=, ch2/Field.h:125-134 */
__global__ void k_density(int64_t nn, const unsigned long long *__restrict__ acc, double unit,
                          const double *__restrict__ vol, const double *__restrict__ ivol, double *den) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    double d = __ll2double_rn((long long)acc[u]) * unit;
    double v = vol[u];
    /* d / v, correctly rounded, from RN(1/v) (the float64 pipe is narrow) */
    den[u] = !zero_bits(v) ? div_rcp(d, v, ivol[u]) : 0.0;
}

struct ChargeArgs {
    int ns;
    const double *den[8];
    double q[8];
};

/* World::computeChargeDensity: rho = 0; rho += den_s * q_s (charged species) */
__global__ void k_charge(int64_t nn, ChargeArgs a, double *rho) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    double r = 0;
    for (int s = 0; s < a.ns; s++) r += a.den[s][u] * a.q[s];
    rho[u] = r;
}

/* Field_::updateAverage */
__global__ void k_update_average(int64_t nn, const double *__restrict__ den, double *ave, int samples) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    ave[u] = (den[u] + samples * ave[u]) / (samples + 1);
}

/* ------------------------------------------------------------------------ */
/* Deterministic reductions: a fixed grid of blocks, fixed per-thread order,
 * fixed tree within the block, partials summed in block order. */
constexpr int RED_BLOCKS = 592, RED_THREADS = 256;

template <int NV>
__device__ __forceinline__ void block_sum_store(double (&v)[NV], double *out) {
    __shared__ double sh[NV][RED_THREADS / 32];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < NV) {
        double s = 0;
        for (int k = 0; k < RED_THREADS / 32; k++) s += sh[threadIdx.x][k];
        out[threadIdx.x] = s;
    }
}

/* per block: {count, mx, my, mz, 2KE/m} of Species::getRealCount/getMomentum/getKE */
template <int FORM>
__global__ void __launch_bounds__(RED_THREADS) k_diag_partials(const double *__restrict__ P,
                                                               const float *__restrict__ vel, int64_t stride,
                                                               const int64_t *__restrict__ d_count, int uniform,
                                                               double w0, double *partials) {
    int64_t n = d_count[0];
    double acc[5] = {0, 0, 0, 0, 0};
    for (int64_t p = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; p < n; p += (int64_t)RED_BLOCKS * RED_THREADS) {
        double w, v0, v1, v2;
        if (FORM == 0) {
            w = uniform ? w0 : P[6 * stride + p];
            v0 = P[3 * stride + p];
            v1 = P[4 * stride + p];
            v2 = P[5 * stride + p];
        } else {
            w = w0;
            v0 = vel[p];
            v1 = vel[stride + p];
            v2 = vel[2 * stride + p];
        }
        acc[0] += w;
        acc[1] += v0 * w;
        acc[2] += v1 * w;
        acc[3] += v2 * w;
        double vv = v0 * v0 + v1 * v1 + v2 * v2;
        acc[4] += w * vv;
    }
    block_sum_store<5>(acc, partials + 5 * blockIdx.x);
}

/* final sums by one warp: lane l adds partials l, l+32, ... in order, then a
 * fixed butterfly; the same bits on every run */
__global__ void k_diag_final(const double *__restrict__ partials, double mass, double *out) {
    int lane = threadIdx.x & 31;
    double s[5] = {0, 0, 0, 0, 0};
    for (int b = lane; b < RED_BLOCKS; b += 32)
        for (int q = 0; q < 5; q++) s[q] += partials[5 * b + q];
    for (int q = 0; q < 5; q++)
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    if (threadIdx.x == 0) {
        out[0] = s[0];
        out[1] = s[1] * mass;
        out[2] = s[2] * mass;
        out[3] = s[3] * mass;
        out[4] = 0.5 * mass * s[4];
    }
}

__global__ void __launch_bounds__(RED_THREADS) k_pe_partials(int64_t nn, const double *__restrict__ ef,
                                                             const double *__restrict__ vol, double *partials) {
    double acc[1] = {0};
    for (int64_t u = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; u < nn; u += (int64_t)RED_BLOCKS * RED_THREADS) {
        double e0 = ef[3 * u], e1 = ef[3 * u + 1], e2 = ef[3 * u + 2];
        double ef2 = e0 * e0 + e1 * e1 + e2 * e2;
        acc[0] += ef2 * vol[u];
    }
    block_sum_store<1>(acc, partials + blockIdx.x);
}

/* 0.5 eps0 times the sum of k_efield4's block partials, in a fixed order */
__global__ void __launch_bounds__(1024) k_pe_sum(const double *__restrict__ part, int64_t n, double *out) {
    __shared__ double ws[32];
    double s = 0;
    for (int64_t b = threadIdx.x; b < n; b += blockDim.x) s += part[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0;
        for (int w32 = 0; w32 < 32; w32++) t += ws[w32];
        out[0] = 0.5 * EPS_0 * t;
    }
}

__global__ void k_pe_final(const double *__restrict__ partials, double *out) {
    int lane = threadIdx.x & 31;
    double s = 0;
    for (int b = lane; b < RED_BLOCKS; b += 32) s += partials[b];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) out[0] = 0.5 * EPS_0 * s;
}

/* ------------------------------------------------------------------------ */
/* Red-black SOR (omega = 1.4) of PotentialSolver::solve over interior nodes,
 * as one cooperative launch: colour c = (i+j+k)&1 holds the nodes updated in
 * half-sweep c; the residual of ch2/PotentialSolver.cpp:44-61 is evaluated
 * every 25 iterations, reduced deterministically and tested by every block. */
__device__ __forceinline__ double grid_sum(cg::grid_group &grid, double v, double *partials, int &round) {
    __shared__ double sh[32];
    __shared__ double total;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double *slot = partials + (round & 1) * gridDim.x;
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[k];
        slot[blockIdx.x] = s;
    }
    round++;
    grid.sync();
    /* every block sums the partials identically: lane l takes l, l+32, ... */
    if (wid == 0) {
        double s = 0;
        for (unsigned b = lane; b < gridDim.x; b += 32) s += __ldcg(slot + b);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        if (lane == 0) total = s;
    }
    __syncthreads();
    return total;
}

struct ColourRange {
    int hx; /* colour nodes per interior row, rounded up */
    int64_t count;
};

__device__ __forceinline__ bool colour_node(const Geo &g, const ColourRange &cr, int64_t t, int c, int &i, int &j,
                                            int &k) {
    int i2 = (int)(t % cr.hx);
    int64_t r = t / cr.hx;
    j = 1 + (int)(r % (g.nj - 2));
    k = 1 + (int)(r / (g.nj - 2));
    i = 1 + 2 * i2 + ((1 + j + k + c) & 1);
    return i <= g.ni - 2;
}

__global__ void __launch_bounds__(256) k_sor_box(Geo g, double *phi, const double *__restrict__ rho, int max_it,
                                                 double tol, double *partials, SolveStatus *st, int *err) {
    cg::grid_group grid = cg::this_grid();
    const double idx2 = 1.0 / (g.dh[0] * g.dh[0]);
    const double idy2 = 1.0 / (g.dh[1] * g.dh[1]);
    const double idz2 = 1.0 / (g.dh[2] * g.dh[2]);
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    ColourRange cr;
    cr.hx = (g.ni - 2 + 1) / 2;
    cr.count = (int64_t)cr.hx * (g.nj - 2) * (g.nk - 2);
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
    const int64_t interior = (int64_t)(g.ni - 2) * (g.nj - 2) * (g.nk - 2);
    double L2 = 0;
    int conv = 0, it, round = 0;
    for (it = 0; it < max_it; it++) {
        for (int c = 0; c < 2; c++) {
            for (int64_t t = gtid; t < cr.count; t += gsize) {
                int i, j, k;
                if (!colour_node(g, cr, t, c, i, j, k)) continue;
                int64_t u = node_of(g, i, j, k);
                double phi_new = (rho[u] / EPS_0 + idx2 * (phi[u - 1] + phi[u + 1]) +
                                  idy2 * (phi[u - sy] + phi[u + sy]) + idz2 * (phi[u - sz] + phi[u + sz])) /
                                 (2 * idx2 + 2 * idy2 + 2 * idz2);
                phi[u] = phi[u] + 1.4 * (phi_new - phi[u]);
            }
            grid.sync();
        }
        if (it % 25 == 0) {
            double sum = 0;
            for (int64_t t = gtid; t < interior; t += gsize) {
                int i = 1 + (int)(t % (g.ni - 2));
                int64_t r = t / (g.ni - 2);
                int j = 1 + (int)(r % (g.nj - 2));
                int k = 1 + (int)(r / (g.nj - 2));
                int64_t u = node_of(g, i, j, k);
                double R = -phi[u] * (2 * idx2 + 2 * idy2 + 2 * idz2) + rho[u] / EPS_0 +
                           idx2 * (phi[u - 1] + phi[u + 1]) + idy2 * (phi[u - sy] + phi[u + sy]) +
                           idz2 * (phi[u - sz] + phi[u + sz]);
                sum += R * R;
            }
            double tot = grid_sum(grid, sum, partials, round);
            L2 = sqrt(tot / ((double)g.ni * g.nj * g.nk));
            if (!isfinite(L2)) {
                if (gtid == 0) atomicOr(err, DERR_NONFINITE);
                break;
            }
            if (L2 < tol) {
                conv = 1;
                break;
            }
        }
    }
    if (gtid == 0) {
        st->converged = conv;
        st->iterations = conv ? it + 1 : it;
        st->inner_iterations = 0;
        st->residual = L2;
        st->solves += 1;
        st->outer_total += st->iterations;
    }
}

/* Red-black form of solveGS: red then black interior non-Dirichlet nodes with
 * the Boltzmann term, then every Neumann node copies the end of its chain. */
__global__ void __launch_bounds__(256) k_gs_sphere(Geo g, double *phi, const double *__restrict__ rho,
                                                   const int32_t *__restrict__ obj,
                                                   const int32_t *__restrict__ target, double phi0, double te0,
                                                   double n0, int max_it, double tol, double *partials,
                                                   SolveStatus *st, int *err) {
    cg::grid_group grid = cg::this_grid();
    const double idx2 = 1.0 / (g.dh[0] * g.dh[0]);
    const double idy2 = 1.0 / (g.dh[1] * g.dh[1]);
    const double idz2 = 1.0 / (g.dh[2] * g.dh[2]);
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    const int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    ColourRange cr;
    cr.hx = (g.ni - 2 + 1) / 2;
    cr.count = (int64_t)cr.hx * (g.nj - 2) * (g.nk - 2);
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
    double L2 = 0;
    int conv = 0, it, round = 0;
    for (it = 0; it < max_it; it++) {
        for (int c = 0; c < 2; c++) {
            for (int64_t t = gtid; t < cr.count; t += gsize) {
                int i, j, k;
                if (!colour_node(g, cr, t, c, i, j, k)) continue;
                int64_t u = node_of(g, i, j, k);
                if (obj[u] > 0) continue;
                double ne = n0 * exp((phi[u] - phi0) / te0);
                double phi_new = ((rho[u] - QE * ne) / EPS_0 + idx2 * (phi[u - 1] + phi[u + 1]) +
                                  idy2 * (phi[u - sy] + phi[u + sy]) + idz2 * (phi[u - sz] + phi[u + sz])) /
                                 (2 * idx2 + 2 * idy2 + 2 * idz2);
                phi[u] = phi[u] + 1.4 * (phi_new - phi[u]);
            }
            grid.sync();
        }
        for (int64_t u = gtid; u < nn; u += gsize) {
            int32_t t = target[u];
            if (t >= 0) phi[u] = phi[t];
        }
        grid.sync();
        if (it % 25 == 0) {
            double sum = 0;
            for (int64_t u = gtid; u < nn; u += gsize) {
                if (obj[u] > 0) continue;
                int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / sz);
                int64_t nb = neumann_next(g, i, j, k);
                double R;
                if (nb >= 0)
                    R = phi[u] - phi[nb];
                else {
                    double ne = n0 * exp((phi[u] - phi0) / te0);
                    R = -phi[u] * (2 * idx2 + 2 * idy2 + 2 * idz2) + (rho[u] - QE * ne) / EPS_0 +
                        idx2 * (phi[u - 1] + phi[u + 1]) + idy2 * (phi[u - sy] + phi[u + sy]) +
                        idz2 * (phi[u - sz] + phi[u + sz]);
                }
                sum += R * R;
            }
            double tot = grid_sum(grid, sum, partials, round);
            L2 = sqrt(tot / ((double)g.ni * g.nj * g.nk));
            if (!isfinite(L2)) {
                if (gtid == 0) atomicOr(err, DERR_NONFINITE);
                break;
            }
            if (L2 < tol) {
                conv = 1;
                break;
            }
        }
    }
    if (gtid == 0) {
        st->converged = conv;
        st->iterations = conv ? it + 1 : it;
        st->inner_iterations = 0;
        st->residual = L2;
        st->solves += 1;
        st->outer_total += st->iterations;
    }
}

/* solveQN: phi = phi0 + Te0 ln(max(rho/rho0, 1e-6)) off the Dirichlet nodes */
__global__ void k_qn(int64_t nn, double *phi, const double *__restrict__ rho, const int32_t *__restrict__ obj,
                     double phi0, double te0, double n0) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn || obj[u] > 0) return;
    double rho0 = n0 * QE;
    double ratio = rho[u] / rho0;
    if (ratio < 1e-6) ratio = 1e-6;
    phi[u] = phi0 + te0 * log(ratio);
}

/* World::computeNodeVolumes, ch2/World.cpp:58-69 */
__global__ void k_node_vol(Geo g, double *vol) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
    double V = g.dh[0] * g.dh[1] * g.dh[2];
    if (i == 0 || i == g.ni - 1) V *= 0.5;
    if (j == 0 || j == g.nj - 1) V *= 0.5;
    if (k == 0 || k == g.nk - 1) V *= 0.5;
    vol[u] = V;
}

/* RN(1 / node_vol) for the density's division (0 where the volume is 0) */
__global__ void k_inv_vol(int64_t nn, const double *__restrict__ vol, double *ivol) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    const double v = vol[u];
    ivol[u] = v != 0 ? 1.0 / v : 0.0;
}

__global__ void k_ef_to_ef4(int64_t nn, const double *__restrict__ ef, float4 *ef4) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    ef4[u] = make_float4((float)ef[3 * u], (float)ef[3 * u + 1], (float)ef[3 * u + 2], 0.f);
}

/* output snapshot: object_id, node_vol, phi, rho, den and den_ave of each
 * species, ef ([nn][3]), one after the other in that order */
struct SnapArgs {
    int ns;
    const double *den[8], *ave[8];
};

__global__ void k_snapshot(int64_t nn, const int32_t *__restrict__ obj, const double *__restrict__ vol,
                           const double *__restrict__ phi, const double *__restrict__ rho,
                           const double *__restrict__ ef, SnapArgs a, double *out) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    out[u] = (double)obj[u];
    out[nn + u] = vol[u];
    out[2 * nn + u] = phi[u];
    out[3 * nn + u] = rho[u];
    for (int s = 0; s < a.ns; s++) {
        out[(4 + s) * nn + u] = a.den[s][u];
        out[(4 + a.ns + s) * nn + u] = a.ave[s][u];
    }
    double *e = out + (4 + 2 * (int64_t)a.ns) * nn;
    e[3 * u] = ef[3 * u];
    e[3 * u + 1] = ef[3 * u + 1];
    e[3 * u + 2] = ef[3 * u + 2];
}

void launch_snapshot(World &w, double *out) {
    SnapArgs a;
    a.ns = (int)w.species.size() < 8 ? (int)w.species.size() : 8;
    for (int s = 0; s < a.ns; s++) {
        a.den[s] = w.species[s]->den;
        a.ave[s] = w.species[s]->den_ave;
    }
    ensure_ef64(w);
    k_snapshot<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, w.obj, w.vol, w.phi, w.rho, w.ef, a, out);
    w.nlaunch++;
}

/* Newton predictor: on the unknowns phi <- 2 phi - phi_prev and phi_prev <-
 * the old phi (extrapolate), or only phi_prev <- phi */
__global__ void k_predict(Geo g, const int32_t *__restrict__ obj, double *phi, double *phi_prev, int extrapolate) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    const double cur = phi[u];
    if (extrapolate && obj[u] == 0) {
        const int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
        if (i > 0 && j > 0 && k > 0 && i < g.ni - 1 && j < g.nj - 1 && k < g.nk - 1) phi[u] = 2.0 * cur - phi_prev[u];
    }
    phi_prev[u] = cur;
}

void launch_predict(World &w, bool extrapolate) {
    k_predict<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.g, w.obj, w.phi, w.phi_prev, extrapolate ? 1 : 0);
    w.nlaunch++;
}

/* weight row of a float64 species that switches from uniform to per-particle weights */
__global__ void k_fill(double *x, int64_t n, double v) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u < n) x[u] = v;
}

/* ======================================================================== */
/* launchers; each adds the number of kernels it launched to w.nlaunch        */
void launch_objects_sphere(World &w, const double c[3], double radius, double phi_s) {
    double4 s = make_double4(c[0], c[1], c[2], radius * radius);
    k_objects_sphere<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.g, s, phi_s, w.obj, w.phi);
    w.nlaunch++;
}

void launch_objects_inlet(World &w) {
    k_objects_inlet<<<blocks_for((int64_t)w.g.ni * w.g.nj, 256), 256, 0, w.stream>>>(w.g, w.obj, w.phi);
    w.nlaunch++;
}

void launch_targets(World &w) {
    k_targets<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.g, w.obj, w.target);
    w.nlaunch++;
}

void launch_efield(World &w, bool full) {
    bool mixed = false, fp64 = false;
    for (Species *s : w.species) {
        mixed |= (s->form == 1);
        fp64 |= (s->form == 0);
    }
    /* RN(1 / (2 dh)) per axis, for div_rcp */
    double3 y2 = make_double3(1.0 / (2 * w.g.dh[0]), 1.0 / (2 * w.g.dh[1]), 1.0 / (2 * w.g.dh[2]));
    dim3 grid((unsigned)blocks_for((int64_t)w.g.ni * w.g.nj, 256), (unsigned)w.g.nk);
    dim3 grid4(grid.x, (unsigned)((w.g.nk + EF_KPT - 1) / EF_KPT));
    const int64_t nparts = (int64_t)grid4.x * grid4.y;
    if (!full && mixed && !fp64 && !w.phi_ef) {
        /* allocated once per world on the first such call */
        if (cudaMalloc(&w.pe_part, nparts * sizeof(double)) != cudaSuccess) w.pe_part = nullptr;
        if (w.pe_part && cudaMalloc(&w.phi_ef, w.nn * sizeof(double)) != cudaSuccess) w.phi_ef = nullptr;
        if (!w.phi_ef && w.pe_part) {
            cudaFree(w.pe_part);
            w.pe_part = nullptr;
        }
    }
    if (!full && mixed && !fp64 && w.phi_ef) {
        EfConst ec;
        ec.y2 = y2;
        ec.d2 = make_double3(2 * w.g.dh[0], 2 * w.g.dh[1], 2 * w.g.dh[2]);
        const double ny[3] = {-y2.x, -y2.y, -y2.z};
        for (int c = 0; c < 3; c++) {
            const float h = (float)ny[c];
            ec.ny[c] = make_float2(h, (float)(ny[c] - (double)h));
        }
        k_efield4<<<grid4, 256, 0, w.stream>>>(w.g, ec, w.phi, w.ef, w.ef4, w.vol, w.pe_part, w.phi_ef);
        w.nlaunch++;
        w.ef4_valid = true;
        w.ef64_valid = false;
        w.pe_parts = nparts;
        return;
    }
    k_efield<<<grid, 256, 0, w.stream>>>(w.g, y2, w.phi, w.ef, mixed ? w.ef4 : nullptr);
    w.nlaunch++;
    w.ef4_valid = mixed;
    w.ef64_valid = true;
    w.pe_parts = 0;
}

void ensure_ef64(World &w) {
    if (w.ef64_valid) return;
    double3 y2 = make_double3(1.0 / (2 * w.g.dh[0]), 1.0 / (2 * w.g.dh[1]), 1.0 / (2 * w.g.dh[2]));
    dim3 grid((unsigned)blocks_for((int64_t)w.g.ni * w.g.nj, 256), (unsigned)w.g.nk);
    /* from the potential of the last computeEF */
    k_efield<<<grid, 256, 0, w.stream>>>(w.g, y2, w.phi_ef, w.ef, nullptr);
    w.nlaunch++;
    w.ef64_valid = true;
}

template <int WALLS, bool DEP, bool UNI>
static void push_fp64_as(World &w, Species &s, int blocks) {
    double sc = w.dt * s.charge / s.mass;
    double4 sph = make_double4(w.sphere[0], w.sphere[1], w.sphere[2], w.has_sphere ? w.sphere[3] : -1.0);
    k_push_fp64<WALLS, DEP, UNI><<<blocks, 256, 0, w.stream>>>(w.g, w.ef, sc, w.dt, s.P, s.cap, s.d_count, sph,
                                                              s.deadmask, s.tiledead, s.acc, s.fx, s.mpw0, w.d_err);
    w.nlaunch++;
}

void launch_push_fp64(World &w, Species &s, bool deposit) {
    int64_t n = s.host_bound;
    if (n <= 0) return;
    ensure_ef64(w);
    int blocks = blocks_for(n, 256);
    if (s.walls == 0) {
        if (!deposit)
            push_fp64_as<REFLECT, false, true>(w, s, blocks);
        else if (s.uniform_w)
            push_fp64_as<REFLECT, true, true>(w, s, blocks);
        else
            push_fp64_as<REFLECT, true, false>(w, s, blocks);
    } else {
        if (!deposit)
            push_fp64_as<ABSORB, false, true>(w, s, blocks);
        else if (s.uniform_w)
            push_fp64_as<ABSORB, true, true>(w, s, blocks);
        else
            push_fp64_as<ABSORB, true, false>(w, s, blocks);
    }
}

void launch_deposit_fp64(World &w, Species &s) {
    int64_t n = s.host_bound;
    if (n <= 0) return;
    if (s.uniform_w)
        k_deposit_fp64<true><<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, s.P, s.cap, s.d_count, s.acc, s.fx,
                                                                       s.mpw0);
    else
        k_deposit_fp64<false><<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, s.P, s.cap, s.d_count, s.acc, s.fx,
                                                                        s.mpw0);
    w.nlaunch++;
}

void launch_compact(World &w, Species &s) {
    if (s.host_bound <= 0) return;
    int64_t ntiles = (s.host_bound + TILE_PARTICLES - 1) / TILE_PARTICLES;
    k_tile_scan<<<1, 1024, 0, w.stream>>>(s.d_count, s.tiledead, s.tilepre);
    int g1 = (int)(ntiles < 2 * (int64_t)w.sm_count ? ntiles : 2 * (int64_t)w.sm_count);
    k_holes<<<g1, 1024, 0, w.stream>>>(s.d_count, s.deadmask, s.tilepre, s.holes);
    int rows = s.uniform_w ? 6 : 7;
    if (s.form == 0)
        k_movers<0><<<g1 * 4, 1024, 0, w.stream>>>(s.d_count, s.deadmask, s.tilepre, s.holes, s.P, nullptr, nullptr,
                                                nullptr, s.cap, rows);
    else
        k_movers<1><<<g1 * 4, 1024, 0, w.stream>>>(s.d_count, s.deadmask, s.tilepre, s.holes, nullptr, s.cell, s.off,
                                                s.vel, s.ms, rows);
    w.nlaunch += 3;
}

void launch_density(World &w, Species &s) {
    k_density<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, s.acc, s.unit, w.vol, w.ivol, s.den);
    w.nlaunch++;
}

void launch_charge(World &w) {
    ChargeArgs a;
    a.ns = 0;
    for (Species *s : w.species) {
        if (s->charge == 0) continue;
        if (a.ns == 8) break;
        a.den[a.ns] = s->den;
        a.q[a.ns] = s->charge;
        a.ns++;
    }
    k_charge<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, a, w.rho);
    w.nlaunch++;
}

void launch_update_average(World &w, Species &s) {
    k_update_average<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, s.den, s.den_ave, s.ave_samples);
    w.nlaunch++;
    s.ave_samples++;
}

template <class Gen>
static void append(World &w, Species &s, const Gen &gen, int64_t ncand, int write_w) {
    if (ncand <= 0) return;
    s.dsum_valid = false; /* the push's diagnostics sums miss the new particles */
    int64_t blocks = (ncand + APPEND_THREADS - 1) / APPEND_THREADS;
    if (blocks > w.blockcnt_cap) {
        if (w.d_blockcnt) {
            cudaStreamSynchronize(w.stream);
            cudaFree(w.d_blockcnt);
        }
        w.blockcnt_cap = blocks + 1024;
        if (cudaMalloc(&w.d_blockcnt, w.blockcnt_cap * sizeof(int32_t)) != cudaSuccess) {
            w.d_blockcnt = nullptr;
            w.blockcnt_cap = 0;
            return;
        }
    }
    double qm = s.charge / s.mass;
    const double3 rdh = make_double3(1.0 / w.g.dh[0], 1.0 / w.g.dh[1], 1.0 / w.g.dh[2]);
    const float qmdt2 = (float)(qm * (0.5 * w.dt));
    /* the mixed form rewinds with the float copy of E; in the float64 form a
     * beam's particles start at z = x0, where the float64 field is always
     * current, and any other generator needs all of it */
    if (s.form != 0) {
        if (!w.ef4_valid) launch_ef4(w);
    } else if (!std::is_same<Gen, GenBeam>::value) {
        ensure_ef64(w);
    }
    k_append_count<Gen><<<(unsigned)blocks, APPEND_THREADS, 0, w.stream>>>(w.g, gen, ncand, w.d_blockcnt);
    k_append_scan<<<1, 1024, 0, w.stream>>>(w.d_blockcnt, blocks, s.d_count, s.cap, w.d_err);
    if (s.form == 0)
        k_append_write<Gen, 0><<<(unsigned)blocks, APPEND_THREADS, 0, w.stream>>>(
            w.g, rdh, gen, ncand, w.d_blockcnt, s.d_count, w.ef, nullptr, qm, w.dt, qmdt2, s.P, nullptr, nullptr,
            nullptr, s.cap, s.cap, write_w);
    else
        k_append_write<Gen, 1><<<(unsigned)blocks, APPEND_THREADS, 0, w.stream>>>(
            w.g, rdh, gen, ncand, w.d_blockcnt, s.d_count, w.ef, w.ef4, qm, w.dt, qmdt2, nullptr, s.cell, s.off,
            s.vel, s.ms, s.cap, 0);
    w.nlaunch += 3;
    s.host_bound += ncand;
    if (s.host_bound > s.cap) s.host_bound = s.cap;
}

void launch_add_fp64(World &w, Species &s, const double *d_pos3, const double *d_vel3, const double *d_w,
                     int64_t n, int rewind) {
    (void)rewind;
    GenHost gh{d_pos3, d_vel3, d_w, s.mpw0};
    append(w, s, gh, n, s.uniform_w ? 0 : 1);
}

void launch_load_box(World &w, Species &s, const double x1[3], const double x2[3], double mpw, int64_t num_mp,
                     const double *d_u, uint64_t stream_id) {
    GenBox gb;
    for (int d = 0; d < 3; d++) {
        gb.x1[d] = x1[d];
        gb.x2[d] = x2[d];
    }
    gb.mpw = mpw;
    gb.u = d_u;
    gb.seed = w.seed;
    gb.stream = stream_id;
    append(w, s, gb, num_mp, s.uniform_w ? 0 : 1);
}

void launch_load_qs(World &w, Species &s, const double x1[3], const double x2[3], double mpw,
                    const int num_mp[3]) {
    GenQS q;
    for (int d = 0; d < 3; d++) {
        q.x1[d] = x1[d];
        q.x2[d] = x2[d];
    }
    q.mpw = mpw;
    q.di = (x2[0] - x1[0]) / (num_mp[0] - 1);
    q.dj = (x2[1] - x1[1]) / (num_mp[1] - 1);
    q.dk = (x2[2] - x1[2]) / (num_mp[2] - 1);
    q.n0 = num_mp[0];
    q.n1 = num_mp[1];
    q.n2 = num_mp[2];
    append(w, s, q, (int64_t)num_mp[0] * num_mp[1] * num_mp[2], s.uniform_w ? 0 : 1);
}

void launch_load_thermal(World &w, Species &s, const double x1[3], const double x2[3], double mpw,
                         int64_t num_mp, const double vd[3], double temp, const double *d_u, uint64_t stream_id) {
    GenThermal g;
    for (int d = 0; d < 3; d++) {
        g.x1[d] = x1[d];
        g.x2[d] = x2[d];
        g.vd[d] = vd[d];
    }
    g.mpw = mpw;
    g.sigma = sqrt(KB * temp / s.mass);
    g.u = d_u;
    g.seed = w.seed;
    g.stream = stream_id;
    append(w, s, g, num_mp, s.uniform_w ? 0 : 1);
}

void launch_inject(World &w, Species &s, int num_sim, double v_drift, double temp, int vmode, const double *d_u,
                   uint64_t stream_id) {
    GenBeam b;
    for (int d = 0; d < 3; d++) b.x0[d] = w.g.x0[d];
    b.Lx = w.g.dh[0] * (w.g.ni - 1);
    b.Ly = w.g.dh[1] * (w.g.nj - 1);
    b.ncx = (double)(w.g.ni - 1);
    b.ncy = (double)(w.g.nj - 1);
    b.dhx = w.g.dh[0];
    b.dhy = w.g.dh[1];
    b.v_drift = v_drift;
    b.mpw0 = s.mpw0;
    b.mode = vmode;
    /* thermal speed: sqrt(2 k T / m) of ch4 (KB) and of ch9/MPI (its own
     * Kb = 1.3806488e-23, ch9/MPI/include/World.h:17); sqrt(k T / m) per
     * component for the Maxwellian */
    b.v_th = vmode == 1 ? sqrt(2 * KB * temp / s.mass)
                        : (vmode == 2 ? sqrt(2 * 1.3806488e-23 * temp / s.mass)
                                      : (vmode == 3 ? sqrt(KB * temp / s.mass) : 0.0));
    b.u = d_u;
    b.seed = w.seed;
    b.stream = stream_id;
    append(w, s, b, num_sim, s.uniform_w ? 0 : 1);
}

void launch_diag(World &w, Species &s, double *d_out5) {
    if (s.form != 0) {
        launch_diag_mixed(w, s, d_out5);
        return;
    }
    k_diag_partials<0><<<RED_BLOCKS, RED_THREADS, 0, w.stream>>>(s.P, nullptr, s.cap, s.d_count, s.uniform_w,
                                                                 s.mpw0, w.d_partials);
    k_diag_final<<<1, 32, 0, w.stream>>>(w.d_partials, s.mass, d_out5);
    w.nlaunch += 2;
}

/* ------------------------------------------------------------------------ */
/* DSMC_MEX (ch4/Collisions.h:51-75, ch4/Collisions.cpp:84-183): neutral-
 * neutral collisions by Bird's no-time-counter scheme with the variable-
 * hard-sphere cross-section, in the float64 form.  Particles are grouped by
 * World::XtoC (ch4/World.h:79-98) with a counting sort (cell and arrival slot
 * per atom, a scan of the cell counts, a scatter); one warp per cell then
 * puts the cell's list in particle order (parts_in_cell) with a bitonic
 * network, and one thread per cell works the pairs, drawing its uniforms in
 * the reference's rnd() order: from a counter-based stream keyed by (call,
 * cell), or, for parity checks, from the caller's array at the cell's offset.
 * Every operation keeps the reference's operand order (unit built with
 * -fmad=false). */
struct DsmcArgs {
    Geo g;
    double mass, Fn, dt, dV, c[4];
    int64_t n_cells;
    const int32_t *count, *start;
    const int32_t *perm;
    double *P;
    int64_t stride;
    unsigned long long *state;
    const double *u;
    int64_t nu;
    const int64_t *cell_off;
    uint64_t seed, stream;
    int *err;
};

/* World::XtoIJK (ch4/World.h:79-92) along one axis without a float64
 * division: x is cut to a float (24 leading bits, by integer operations so
 * that nothing queues on the narrow float64 pipe), q = (x_f - x0_f) / dh in
 * float, and q's integer part is the reference's (int)((x - x0) / dh)
 * whenever q lies farther than tol from an integer; tol bounds the error of
 * the float estimate (host side, dsmc_axis).  Anything else (near a cell
 * face, outside the grid, huge or not finite) takes the float64 division. */
struct DsmcAxis {
    float x0f, invf, tol;
    int nc;
};

__device__ __forceinline__ int dsmc_coord(double x, double x0, double dh, DsmcAxis ax) {
    const int hi = __double2hiint(x);
    const unsigned lo = (unsigned)__double2loint(x);
    const int fe = ((hi >> 20) & 0x7ff) - 896; /* float exponent field */
    float xf = 0.0f;                            /* |x| < 2^-126: zero */
    if (fe >= 1) xf = __int_as_float((hi & (int)0x80000000) | (fe << 23) | ((hi & 0xfffff) << 3) | (int)(lo >> 29));
    const float q = (xf - ax.x0f) * ax.invf;
    if (fe <= 254 && q >= 0.0f && q < (float)ax.nc) {
        const int k = (int)q;
        const float fr = q - (float)k; /* exact: k <= q < k + 1 */
        if (fr > ax.tol && fr < 1.0f - ax.tol) return k;
    }
    return (int)((x - x0) / dh);
}

static DsmcAxis dsmc_axis(double x0, double xm, double dh, int nc) {
    /* |q - (x - x0)/dh| <= 2^-23 |x| / dh + 2^-24 |x0| / dh (x and x0 to
     * float) + 3 roundings of 2^-24 relative on q (the subtraction, 1/dh,
     * the product) for 0 <= q < nc; doubled, plus the float64 quotient's
     * own rounding */
    const double L = fmax(fabs(x0), fabs(xm)) + dh;
    const double err = 3.01 * ldexp(1.0, -24) * (nc + 1.0) + (ldexp(1.0, -23) * L + ldexp(1.0, -24) * fabs(x0)) / dh;
    const double tol = 2 * err + 1e-12;
    DsmcAxis a;
    a.x0f = (float)x0;
    a.invf = (float)(1.0 / dh);
    a.tol = tol < 0.01 ? (float)tol : 2.0f; /* 2: always the division */
    a.nc = nc;
    return a;
}

/* each atom's cell and its slot among the cell's atoms (arrival order) */
__global__ void k_dsmc_cells(Geo g, DsmcAxis ax, DsmcAxis ay, DsmcAxis az, const double *__restrict__ P,
                             int64_t stride, const int64_t *__restrict__ d_count, int64_t n_cells, int32_t *cell,
                             int32_t *rank, int32_t *count, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d_count[0]) return;
    const int i = dsmc_coord(P[p], g.x0[0], g.dh[0], ax);
    const int j = dsmc_coord(P[stride + p], g.x0[1], g.dh[1], ay);
    const int k = dsmc_coord(P[2 * stride + p], g.x0[2], g.dh[2], az);
    const int64_t c = (int64_t)k * (g.nj - 1) * (g.ni - 1) + (int64_t)j * (g.ni - 1) + i;
    const bool in = i >= 0 && j >= 0 && k >= 0 && i < g.ni - 1 && j < g.nj - 1 && k < g.nk - 1 && c < n_cells;
    if (!in) {
        atomicOr(err, DERR_DSMC);
        cell[p] = -1;
        return;
    }
    cell[p] = (int32_t)c;
    rank[p] = atomicAdd(count + c, 1);
}

__global__ void k_dsmc_scatter(const int32_t *__restrict__ cell, const int32_t *__restrict__ rank,
                               const int64_t *__restrict__ d_count, const int32_t *__restrict__ start,
                               int32_t *perm) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d_count[0]) return;
    const int32_t c = cell[p];
    if (c < 0) return;
    perm[start[c] + rank[p]] = (int32_t)p;
}

/* Bitonic sort of 32 R values held R per lane (element i*32 + lane in a[i]),
 * ascending: exchanges between lanes by shuffles, within a lane by swaps. */
template <int R>
__device__ __forceinline__ void warp_bitonic(int32_t (&a)[R], int lane) {
#pragma unroll
    for (int k = 2; k <= 32 * R; k <<= 1) {
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= 32) {
                const int jj = j >> 5;
#pragma unroll
                for (int i = 0; i < R; i++) {
                    if ((i & jj) == 0) {
                        const bool up = ((i * 32 + lane) & k) == 0;
                        const int32_t x = a[i], y = a[i | jj];
                        const bool sw = up ? (x > y) : (x < y);
                        a[i] = sw ? y : x;
                        a[i | jj] = sw ? x : y;
                    }
                }
            } else {
#pragma unroll
                for (int i = 0; i < R; i++) {
                    const int32_t y = __shfl_xor_sync(0xffffffffu, a[i], j);
                    const bool lower = (lane & j) == 0;
                    const bool up = ((i * 32 + lane) & k) == 0;
                    a[i] = (lower == up) ? min(a[i], y) : max(a[i], y);
                }
            }
        }
    }
}

template <int R>
__device__ __forceinline__ void order_segment(int32_t *parts, int np, int lane) {
    int32_t a[R];
#pragma unroll
    for (int i = 0; i < R; i++) a[i] = i * 32 + lane < np ? parts[i * 32 + lane] : INT_MAX;
    warp_bitonic<R>(a, lane);
#pragma unroll
    for (int i = 0; i < R; i++)
        if (i * 32 + lane < np) parts[i * 32 + lane] = a[i];
}

/* each cell's atoms in particle order (the order of parts_in_cell,
 * ch4/Collisions.cpp:116-121): one warp per cell */
__global__ void __launch_bounds__(256) k_dsmc_order(const int32_t *__restrict__ count,
                                                    const int32_t *__restrict__ start, int32_t *perm,
                                                    int64_t n_cells) {
    const int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (c >= n_cells) return; /* whole warps */
    const int np = count[c];
    if (np < 2) return;
    int32_t *parts = perm + start[c];
    if (np <= 32) order_segment<1>(parts, np, lane);
    else if (np <= 64) order_segment<2>(parts, np, lane);
    else if (np <= 128) order_segment<4>(parts, np, lane);
    else if (np <= 256) order_segment<8>(parts, np, lane);
    else if (np <= 512) order_segment<16>(parts, np, lane);
    else if (np <= 1024) order_segment<32>(parts, np, lane);
    else if (lane == 0) {
        for (int i = 1; i < np; i++) {
            const int32_t v = parts[i];
            int j = i - 1;
            while (j >= 0 && parts[j] > v) {
                parts[j + 1] = parts[j];
                j--;
            }
            parts[j + 1] = v;
        }
    }
}

__global__ void k_dsmc_begin(unsigned long long *state) {
    state[1] = 0ull;
    state[2] = 0ull;
}

/* sqrt of ((0 + x x) + y y) + z z, vec3 mag of ch4/Field.h:21-26 */
__device__ __forceinline__ double dsmc_mag(double x, double y, double z) {
    double s = 0;
    s += x * x;
    s += y * y;
    s += z * z;
    return sqrt(s);
}

__global__ void __launch_bounds__(128) k_dsmc_collide(DsmcArgs a) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.n_cells) return;
    const int np = a.count[c];
    if (np < 2) return;
    const int32_t *parts = a.perm + a.start[c]; /* in particle order */
    const double smax = __longlong_as_double((long long)a.state[0]);
    const double ng_f = 0.5 * np * np * a.Fn * smax * a.dt / a.dV;
    const int ng = (int)(ng_f + 0.5);
    const double *u = a.u ? a.u + a.cell_off[c] : nullptr;
    const int64_t ulim = a.u ? a.nu - a.cell_off[c] : 0;
    int64_t k = 0;
    bool short_u = false;
    auto U = [&]() -> double {
        if (u) {
            if (k >= ulim) {
                short_u = true;
                return 0.5;
            }
            return u[k++];
        }
        return philox_uniform(a.seed, a.stream, ((uint64_t)c << 32) + (uint64_t)(k++));
    };
    double local_max = 0;
    unsigned long long cols = 0;
    double *V = a.P + 3 * a.stride;
    for (int gg = 0; gg < ng && !short_u; gg++) {
        const int p1 = (int)(U() * np);
        int p2;
        do {
            p2 = (int)(U() * np);
        } while (p2 == p1 && !short_u);
        if (short_u) break;
        const int64_t i1 = parts[p1], i2 = parts[p2];
        const double cr = dsmc_mag(V[i1] - V[i2], V[a.stride + i1] - V[a.stride + i2],
                                   V[2 * a.stride + i1] - V[2 * a.stride + i2]);
        /* DSMC_MEX::evalSigma, ch4/Collisions.h:64-67 */
        const double sigma = REF_PI * a.c[0] * a.c[0] * pow(a.c[2] / (cr * cr), a.c[1] - 0.5) / a.c[3];
        const double sigma_cr = sigma * cr;
        if (sigma_cr > local_max) local_max = sigma_cr;
        const double Pc = sigma_cr / smax;
        if (Pc > U()) {
            const double u_chi = U(), u_eps = U();
            if (short_u) break;
            cols++;
            /* DSMC_MEX::collide, ch4/Collisions.cpp:84-105 */
            const double m1 = a.mass, m2 = a.mass;
            double v1[3], v2[3], cm[3], crv[3];
            for (int d = 0; d < 3; d++) {
                v1[d] = V[d * a.stride + i1];
                v2[d] = V[d * a.stride + i2];
            }
            for (int d = 0; d < 3; d++) cm[d] = (v1[d] * m1 + v2[d] * m2) / (m1 + m2);
            for (int d = 0; d < 3; d++) crv[d] = v1[d] - v2[d];
            const double cr_mag = dsmc_mag(crv[0], crv[1], crv[2]);
            const double cos_chi = 2 * u_chi - 1;
            const double sin_chi = sqrt(1 - cos_chi * cos_chi);
            const double eps = 2 * REF_PI * u_eps;
            crv[0] = cr_mag * cos_chi;
            crv[1] = cr_mag * sin_chi * cos(eps);
            crv[2] = cr_mag * sin_chi * sin(eps);
            const double s1 = m2 / (m1 + m2), s2 = m1 / (m1 + m2);
            for (int d = 0; d < 3; d++) {
                V[d * a.stride + i1] = cm[d] + crv[d] * s1;
                V[d * a.stride + i2] = cm[d] - crv[d] * s2;
            }
        }
    }
    if (short_u) atomicOr(a.err, DERR_DSMC);
    /* sigma*cr >= 0: the order of the bit patterns is the order of the values */
    if (local_max > 0) atomicMax(a.state + 1, (unsigned long long)__double_as_longlong(local_max));
    if (cols) atomicAdd(a.state + 2, cols);
}

/* sigma_cr_max takes the call's largest sigma*cr when a collision happened */
__global__ void k_dsmc_finish(unsigned long long *state) {
    if (state[2]) state[0] = state[1];
    state[3] += state[2];
}

void launch_dsmc(World &w, Species &s, double dt, const double *d_u, int64_t nu, const int64_t *d_cell_off) {
    const int64_t n = s.host_bound;
    const int64_t n_cells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    const DsmcAxis ax = dsmc_axis(w.g.x0[0], w.g.xm[0], w.g.dh[0], w.g.ni - 1);
    const DsmcAxis ay = dsmc_axis(w.g.x0[1], w.g.xm[1], w.g.dh[1], w.g.nj - 1);
    const DsmcAxis az = dsmc_axis(w.g.x0[2], w.g.xm[2], w.g.dh[2], w.g.nk - 1);
    cudaMemsetAsync(s.dsmc_count, 0, (n_cells + 1) * sizeof(int32_t), w.stream);
    if (n > 0)
        k_dsmc_cells<<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, ax, ay, az, s.P, s.cap, s.d_count, n_cells,
                                                                s.dsmc_cell, s.dsmc_rank, s.dsmc_count, w.d_err);
    cudaMemcpyAsync(s.dsmc_start, s.dsmc_count, (n_cells + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                    w.stream);
    launch_int_excl_scan(w.stream, s.dsmc_start, n_cells, s.dsmc_bsum);
    if (n > 0)
        k_dsmc_scatter<<<blocks_for(n, 256), 256, 0, w.stream>>>(s.dsmc_cell, s.dsmc_rank, s.d_count,
                                                                  s.dsmc_start, s.dsmc_perm);
    k_dsmc_order<<<blocks_for(n_cells * 32, 256), 256, 0, w.stream>>>(s.dsmc_count, s.dsmc_start, s.dsmc_perm,
                                                                       n_cells);
    k_dsmc_begin<<<1, 1, 0, w.stream>>>(s.d_dsmc);
    DsmcArgs a;
    a.g = w.g;
    a.mass = s.mass;
    a.Fn = s.mpw0;
    a.dt = dt;
    a.dV = w.g.dh[0] * w.g.dh[1] * w.g.dh[2];
    for (int d = 0; d < 4; d++) a.c[d] = s.dsmc_c[d];
    a.n_cells = n_cells;
    a.count = s.dsmc_count;
    a.start = s.dsmc_start;
    a.perm = s.dsmc_perm;
    a.P = s.P;
    a.stride = s.cap;
    a.state = s.d_dsmc;
    a.u = d_u;
    a.nu = nu;
    a.cell_off = d_cell_off;
    a.seed = w.seed;
    /* one stream per (species, call); cell c draws index (c << 32) + k */
    a.stream = (0xD5ull << 56) | ((uint64_t)(s.id & 0xff) << 48) | (s.dsmc_calls & 0xffffffffffffull);
    a.err = w.d_err;
    k_dsmc_collide<<<blocks_for(n_cells, 128), 128, 0, w.stream>>>(a);
    k_dsmc_finish<<<1, 1, 0, w.stream>>>(s.d_dsmc);
    w.nlaunch += 7 + 3;
    s.dsmc_calls++;
}

void launch_pe(World &w, double *d_out1) {
    if (w.pe_parts > 0) { /* the sum k_efield4 left behind */
        k_pe_sum<<<1, 1024, 0, w.stream>>>(w.pe_part, w.pe_parts, d_out1);
        w.nlaunch++;
        return;
    }
    ensure_ef64(w);
    k_pe_partials<<<RED_BLOCKS, RED_THREADS, 0, w.stream>>>(w.nn, w.ef, w.vol, w.d_partials);
    k_pe_final<<<1, 32, 0, w.stream>>>(w.d_partials, d_out1);
    w.nlaunch += 2;
}

static int coop_grid(World &w, const void *fn, int threads, int64_t work) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t maxb = (int64_t)per_sm * w.sm_count;
    int64_t need = (work + threads - 1) / threads;
    if (need < 1) need = 1;
    int g = (int)(need < maxb ? need : maxb);
    if (g > w.partial_slots / 2) g = w.partial_slots / 2;
    if (w.solver_blocks > 0 && g > w.solver_blocks) g = w.solver_blocks;
    return g;
}

int launch_sor_box(World &w, int max_it, double tol) {
    int64_t work = (int64_t)((w.g.ni - 1) / 2) * (w.g.nj - 2) * (w.g.nk - 2);
    int grid = coop_grid(w, (const void *)k_sor_box, 256, work);
    Geo g = w.g;
    double *phi = w.phi;
    const double *rho = w.rho;
    double *part = w.d_partials;
    SolveStatus *st = w.d_status;
    int *err = w.d_err;
    void *args[] = {&g, &phi, &rho, &max_it, &tol, &part, &st, &err};
    w.nlaunch++;
    return (int)cudaLaunchCooperativeKernel((const void *)k_sor_box, grid, 256, args, 0, w.stream);
}

int launch_gs_sphere(World &w, int max_it, double tol) {
    int64_t work = (int64_t)((w.g.ni - 1) / 2) * (w.g.nj - 2) * (w.g.nk - 2);
    int grid = coop_grid(w, (const void *)k_gs_sphere, 256, work);
    Geo g = w.g;
    double *phi = w.phi;
    const double *rho = w.rho;
    const int32_t *obj = w.obj, *tg = w.target;
    double phi0 = w.phi0, te0 = w.te0, n0 = w.n0;
    double *part = w.d_partials;
    SolveStatus *st = w.d_status;
    int *err = w.d_err;
    void *args[] = {&g, &phi, &rho, &obj, &tg, &phi0, &te0, &n0, &max_it, &tol, &part, &st, &err};
    w.nlaunch++;
    return (int)cudaLaunchCooperativeKernel((const void *)k_gs_sphere, grid, 256, args, 0, w.stream);
}

void launch_inv_vol(World &w) {
    k_inv_vol<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, w.vol, w.ivol);
    w.nlaunch++;
}

void launch_node_vol(World &w) {
    k_node_vol<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.g, w.vol);
    launch_inv_vol(w);
    w.nlaunch++;
}

void launch_ef4(World &w) {
    ensure_ef64(w);
    k_ef_to_ef4<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, w.ef, w.ef4);
    w.nlaunch++;
    w.ef4_valid = true;
}

void launch_fill(World &w, double *x, int64_t n, double v) {
    if (n <= 0) return;
    k_fill<<<blocks_for(n, 256), 256, 0, w.stream>>>(x, n, v);
    w.nlaunch++;
}

void launch_qn(World &w) {
    k_qn<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, w.phi, w.rho, w.obj, w.phi0, w.te0, w.n0);
    w.nlaunch++;
}

/* ------------------------------------------------------------------------ */
/* ch4 species moments (float64 form): Species::sampleMoments,
 * computeGasProperties, computeMPC, clearSamples (ch4/Species.cpp:191-240).
 * The seven sampled sums (n, n u, n v, n w, n u u, n v v, n w w) are
 * scattered with the CIC corner weights, each product value * weight rounded
 * once to a 64-bit integer count of 2^-S_q and added exactly (order
 * independent, deterministic); S_q is chosen per call from the call's
 * largest |value| and particle count so that no node can overflow, and each
 * call's integer sums are folded into float64 accumulators. */
/* w0 > 0: every particle carries w0 and the weight row is not stored */
__device__ __forceinline__ void mom_values(const double *__restrict__ P, int64_t stride, int64_t p, double w0,
                                           double v[NMOM]) {
    const double w = w0 > 0 ? w0 : P[6 * stride + p];
    const double u = P[3 * stride + p], vv = P[4 * stride + p], ww = P[5 * stride + p];
    v[0] = w;
    v[1] = w * u;
    v[2] = w * vv;
    v[3] = w * ww;
    v[4] = w * u * u;
    v[5] = w * vv * vv;
    v[6] = w * ww * ww;
}

/* largest |value| of each sum over the particles, as float64 bits (the bits
 * of non-negative values order like the values: integer max, no float64) */
__global__ void __launch_bounds__(256) k_mom_bound(const double *__restrict__ P, int64_t stride, double w0,
                                                   const int64_t *__restrict__ d_count, unsigned long long *bound) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long b[NMOM];
    for (int q = 0; q < NMOM; q++) b[q] = 0;
    if (p < d_count[0]) {
        double v[NMOM];
        mom_values(P, stride, p, w0, v);
        for (int q = 0; q < NMOM; q++) b[q] = (unsigned long long)__double_as_longlong(v[q]) & 0x7fffffffffffffffull;
    }
    for (int q = 0; q < NMOM; q++) {
        unsigned long long x = b[q];
        for (int o = 16; o; o >>= 1) {
            const unsigned long long y = __shfl_xor_sync(0xffffffffu, x, o);
            x = y > x ? y : x;
        }
        if ((threadIdx.x & 31) == 0 && x) atomicMax(bound + q, x);
    }
}

/* scale[q] = 2^S_q with count * max_q * 2^S_q < 2^62 (no node overflows)
 * and max_q * 2^S_q < 2^51 (each product converts by one FMA, see
 * fix_round); scale[NMOM + q] = 2^-S_q */
__global__ void k_mom_scale(const unsigned long long *bound, const int64_t *d_count, double *scale, int *err) {
    const int q = threadIdx.x;
    if (q >= NMOM) return;
    const double b = __longlong_as_double((long long)bound[q]);
    const double t = b * (double)(d_count[0] > 0 ? d_count[0] : 1);
    int S = 0;
    if (!isfinite(t)) {
        atomicOr(err, DERR_NEUTRAL);
    } else if (t > 0) {
        int e, em;
        frexp(t, &e);  /* t < 2^e */
        frexp(b, &em); /* b < 2^em */
        S = 62 - e < 51 - em ? 62 - e : 51 - em;
        S = S > 1000 ? 1000 : (S < -1000 ? -1000 : S);
    }
    scale[q] = ldexp(1.0, S);
    scale[NMOM + q] = ldexp(1.0, -S);
}

/* RN(a b) as a 64-bit integer for |a b| < 2^51: adding 1.5 * 2^52 inside one
 * FMA puts the exact product's nearest integer (ties to even) in the low
 * bits of a number in [2^52, 2^53), whose bit pattern then differs from the
 * constant's by that integer (one float64 operation instead of a product and
 * a conversion) */
__device__ __forceinline__ long long fix_round(double a, double b) {
    const double magic = 6755399441055744.0;
    return __double_as_longlong(__fma_rn(a, b, magic)) - __double_as_longlong(magic);
}

/* corner weights (1-di)(1-dj)(1-dk), di(1-dj)(1-dk), ... in Field_::scatter's
 * corner order (ch4/Field.h:212-232), the dj, dk factors shared */
__device__ __forceinline__ void corner_weights(double di, double dj, double dk, double W[8]) {
    const double a0 = (1 - di) * (1 - dj), a1 = di * (1 - dj), a2 = di * dj, a3 = (1 - di) * dj;
    W[0] = a0 * (1 - dk);
    W[1] = a1 * (1 - dk);
    W[2] = a2 * (1 - dk);
    W[3] = a3 * (1 - dk);
    W[4] = a0 * dk;
    W[5] = a1 * dk;
    W[6] = a2 * dk;
    W[7] = a3 * dk;
}

/* each sum's 8 corner contributions value * W_m, rounded once (from the exact
 * product) to a count of 2^-S_q and added exactly; within one weight
 * rounding of the reference's left-to-right product */
__global__ void __launch_bounds__(256) k_mom_scatter(Geo g, double3 rdh, const double *__restrict__ P, int64_t stride,
                                                     double w0, const int64_t *__restrict__ d_count,
                                                     const double *__restrict__ scale, unsigned long long *acc,
                                                     int64_t nn, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d_count[0]) return;
    const double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
    double lc[3];
    xtol_rcp(g, rdh, x, lc);
    if (!(lc[0] >= 0 && lc[1] >= 0 && lc[2] >= 0 && lc[0] <= g.ni - 1 && lc[1] <= g.nj - 1 && lc[2] <= g.nk - 1)) {
        atomicOr(err, DERR_NEUTRAL);
        return;
    }
    const int i = clamp_cell((int)lc[0], g.ni), j = clamp_cell((int)lc[1], g.nj), k = clamp_cell((int)lc[2], g.nk);
    double W[8];
    corner_weights(lc[0] - i, lc[1] - j, lc[2] - k, W);
    const int64_t n0 = node_of(g, i, j, k), sy = g.ni, sz = (int64_t)g.ni * g.nj;
    const int64_t idx[8] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy, n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
    double v[NMOM];
    mom_values(P, stride, p, w0, v);
#pragma unroll
    for (int q = 0; q < NMOM; q++) {
        const double vf = v[q] * scale[q]; /* exact: a power of two */
        unsigned long long *a = acc + q * nn;
#pragma unroll
        for (int m = 0; m < 8; m++) {
            const long long c = fix_round(vf, W[m]);
            if (c) atomicAdd(a + idx[m], (unsigned long long)c);
        }
    }
}

/* the call's exact integer sums into the float64 accumulators */
__global__ void __launch_bounds__(256) k_mom_fold(int64_t nn, unsigned long long *acc, const double *scale,
                                                  double *mom) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= NMOM * nn) return;
    const int q = (int)(t / nn);
    const long long c = (long long)acc[t];
    if (c) {
        mom[t] += (double)c * scale[NMOM + q];
        acc[t] = 0;
    }
}

/* Species::computeGasProperties (ch4/Species.cpp:204-225): stream velocity
 * nv/n (0 where n == 0, Field_ operator/ at ch4/Field.h:182-196) and
 * T = m / (2 K) ((uu + vv) + ww) with uu = <u u> - u u (0 where n <= 0) */
__global__ void __launch_bounds__(256) k_gas_props(int64_t nn, double mass, const double *__restrict__ mom,
                                                   double *vel, double *T) {
    const int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (u >= nn) return;
    const double count = mom[u];
    double ave[3];
    for (int d = 0; d < 3; d++) {
        ave[d] = count != 0 ? mom[(1 + d) * nn + u] / count : 0.0;
        vel[3 * u + d] = ave[d];
    }
    if (count <= 0) {
        T[u] = 0;
        return;
    }
    const double uu = mom[4 * nn + u] / count - ave[0] * ave[0];
    const double vv = mom[5 * nn + u] / count - ave[1] * ave[1];
    const double ww = mom[6 * nn + u] / count - ave[2] * ave[2];
    T[u] = mass / (2 * KB) * (uu + vv + ww);
}

/* Species::computeMPC (ch4/Species.cpp:228-235): macroparticles per cell
 * (World::XtoIJK); counts below 2^53 are exact in float64 */
__global__ void __launch_bounds__(256) k_mpc(Geo g, const double *__restrict__ P, int64_t stride,
                                             const int64_t *__restrict__ d_count, double *mpc, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d_count[0]) return;
    const double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
    double lc[3];
    xtol(g, x, lc);
    const int i = (int)lc[0], j = (int)lc[1], k = (int)lc[2];
    if (!(lc[0] >= 0 && lc[1] >= 0 && lc[2] >= 0 && i < g.ni - 1 && j < g.nj - 1 && k < g.nk - 1)) {
        atomicOr(err, DERR_NEUTRAL);
        return;
    }
    atomicAdd(mpc + ((int64_t)k * (g.nj - 1) + j) * (g.ni - 1) + i, 1.0);
}

/* MCC_CEX::apply (ch4/Collisions.cpp:43-80): each source particle meets
 * the target gas (density and stream velocity gathered at its position)
 * with probability 1 - exp(-n sigma |v - v_t| dt), sigma = 1e-16 m^2, and
 * then stops (the reference sets vel = 0; its sampled target velocity is
 * never used, so it is not drawn).  One uniform per particle: index p of
 * the call's counter-based stream, or u[p_off[p]] when replaying.  The
 * gathers share one set of corner weights and accumulate with FMAs, so n and
 * v_t lie within a few ulps of the reference's left-to-right sums; a
 * decision can differ only for a uniform within those ulps of the
 * probability. */
__global__ void __launch_bounds__(256) k_mcc_cex(Geo g, double3 rdh, double *P, int64_t stride,
                                                 const int64_t *__restrict__ d_count, const double *__restrict__ den,
                                                 const double *__restrict__ vel, double dt, const double *__restrict__ u,
                                                 int64_t nu, const int64_t *__restrict__ p_off, uint64_t seed,
                                                 uint64_t stream, unsigned long long *ncol, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool hit = false;
    if (p < d_count[0]) {
        const double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double lc[3];
        xtol_rcp(g, rdh, x, lc);
        if (!(lc[0] >= 0 && lc[1] >= 0 && lc[2] >= 0 && lc[0] <= g.ni - 1 && lc[1] <= g.nj - 1 &&
              lc[2] <= g.nk - 1)) {
            atomicOr(err, DERR_NEUTRAL);
        } else {
            const int i = clamp_cell((int)lc[0], g.ni), j = clamp_cell((int)lc[1], g.nj),
                      k = clamp_cell((int)lc[2], g.nk);
            double W[8];
            corner_weights(lc[0] - i, lc[1] - j, lc[2] - k, W);
            const int64_t n0 = node_of(g, i, j, k), sy = g.ni, sz = (int64_t)g.ni * g.nj;
            const int64_t idx[8] = {n0,      n0 + 1,      n0 + 1 + sy,      n0 + sy,
                                    n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
            double nn = 0, vt0 = 0, vt1 = 0, vt2 = 0;
#pragma unroll
            for (int m = 0; m < 8; m++) {
                nn = __fma_rn(den[idx[m]], W[m], nn);
                vt0 = __fma_rn(vel[3 * idx[m]], W[m], vt0);
                vt1 = __fma_rn(vel[3 * idx[m] + 1], W[m], vt1);
                vt2 = __fma_rn(vel[3 * idx[m] + 2], W[m], vt2);
            }
            const double v_rel_mag = dsmc_mag(P[3 * stride + p] - vt0, P[4 * stride + p] - vt1,
                                              P[5 * stride + p] - vt2);
            const double sigma = 1e-16;
            const double Pc = 1 - exp(-nn * sigma * v_rel_mag * dt);
            double U;
            if (u) {
                const int64_t o = p_off[p];
                if (o < 0 || o >= nu) {
                    atomicOr(err, DERR_NEUTRAL);
                    U = 2.0;
                } else {
                    U = u[o];
                }
            } else {
                U = philox_uniform(seed, stream, (uint64_t)p);
            }
            if (Pc >= U) {
                hit = true;
                P[3 * stride + p] = 0;
                P[4 * stride + p] = 0;
                P[5 * stride + p] = 0;
            }
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(ncol, (unsigned long long)__popc(m));
}

static double3 rcp_dh(const World &w) {
    return make_double3(1.0 / w.g.dh[0], 1.0 / w.g.dh[1], 1.0 / w.g.dh[2]);
}

void launch_moments(World &w, Species &s) {
    const int64_t n = s.host_bound;
    cudaMemsetAsync(s.mom_bound, 0, NMOM * sizeof(unsigned long long), w.stream);
    const double w0 = s.uniform_w ? s.mpw0 : 0.0;
    if (n > 0) k_mom_bound<<<blocks_for(n, 256), 256, 0, w.stream>>>(s.P, s.cap, w0, s.d_count, s.mom_bound);
    k_mom_scale<<<1, 32, 0, w.stream>>>(s.mom_bound, s.d_count, s.mom_scale, w.d_err);
    if (n > 0)
        k_mom_scatter<<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, rcp_dh(w), s.P, s.cap, w0, s.d_count,
                                                                 s.mom_scale, s.mom_acc, w.nn, w.d_err);
    k_mom_fold<<<blocks_for(NMOM * w.nn, 256), 256, 0, w.stream>>>(w.nn, s.mom_acc, s.mom_scale, s.mom);
    w.nlaunch += 2 + 2 * (n > 0);
}

void launch_gas_props(World &w, Species &s) {
    k_gas_props<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.nn, s.mass, s.mom, s.gvel, s.gtemp);
    w.nlaunch++;
}

void launch_mpc(World &w, Species &s) {
    const int64_t n = s.host_bound;
    const int64_t n_cells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    cudaMemsetAsync(s.mpc, 0, n_cells * sizeof(double), w.stream);
    if (n > 0) {
        k_mpc<<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, s.P, s.cap, s.d_count, s.mpc, w.d_err);
        w.nlaunch++;
    }
}

void launch_mcc(World &w, Species &src, const Species &tgt, double dt, const double *d_u, int64_t nu,
                const int64_t *d_off, unsigned long long *d_ncol) {
    const int64_t n = src.host_bound;
    cudaMemsetAsync(d_ncol, 0, sizeof(unsigned long long), w.stream);
    if (n > 0) {
        /* one stream per (species, call); particle p draws index p */
        const uint64_t stream = (0xCEull << 56) | ((uint64_t)(src.id & 0xff) << 48) |
                                (src.mcc_calls & 0xffffffffffffull);
        k_mcc_cex<<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, rcp_dh(w), src.P, src.cap, src.d_count, tgt.den,
                                                             tgt.gvel, dt, d_u, nu, d_off, w.seed, stream, d_ncol,
                                                             w.d_err);
        w.nlaunch++;
    }
    src.mcc_calls++;
}

/* ------------------------------------------------------------------------ */
/* ch4 neutral push (ch4_push.h): one thread per particle; particles that
 * leave the domain go to the dead mask and the compaction of the other
 * pushes removes them (the reference's swap-with-last order is not kept;
 * same survivors).  Time of each particle: pdt[p] + dt when the caller gives
 * the particles' time left, else 2 dt for particles appended since the last
 * call (a source's addParticle leaves them one dt, ch4/Species.h:65) and dt
 * for the others.  Uniforms: u[p_off[p] + k] when replaying, else index
 * (p << 10) + k of the call's counter-based stream (k < 715). */
struct Ch4Uniforms {
    const double *u;
    int64_t nu, base;
    uint64_t seed, stream, index0;
    bool bad;
    __device__ double operator()(int k) {
        if (u) {
            const int64_t o = base + k;
            if (o < 0 || o >= nu) {
                bad = true;
                return 0.5;
            }
            return u[o];
        }
        return philox_uniform(seed, stream, index0 + (uint64_t)k);
    }
};

__global__ void __launch_bounds__(256) k_advance_ch4(Ch4Geo G, double mass, double dt, double *P, int64_t stride,
                                                     const int64_t *__restrict__ d_count,
                                                     const int64_t *__restrict__ d_settled,
                                                     const double *__restrict__ pdt, const double *__restrict__ u,
                                                     int64_t nu, const int64_t *__restrict__ p_off, uint64_t seed,
                                                     uint64_t stream, uint32_t *deadmask, int32_t *tiledead,
                                                     unsigned long long *nbounce, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = d_count[0];
    bool dead = false;
    int b = 0;
    if (p < n) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        const double t = (pdt ? pdt[p] : (p >= d_settled[0] ? dt : 0.0)) + dt;
        Ch4Uniforms U{u, nu, u ? p_off[p] : 0, seed, stream, (uint64_t)p << 10, false};
        bool alive = true;
        b = ch4_advance_one(G, mass, t, x, v, U, alive, 64);
        if (U.bad) atomicOr(err, DERR_NEUTRAL);
        if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) {
            atomicOr(err, DERR_NONFINITE);
            alive = false;
        }
        dead = !alive;
        for (int d = 0; d < 3; d++) {
            P[d * stride + p] = x[d];
            P[(3 + d) * stride + p] = v[d];
        }
    }
    const unsigned m = __ballot_sync(0xffffffffu, dead);
    int bs = b;
    for (int o = 16; o; o >>= 1) bs += __shfl_xor_sync(0xffffffffu, bs, o);
    if ((threadIdx.x & 31) == 0 && p < n) {
        deadmask[p >> 5] = m;
        if (m) atomicAdd(tiledead + (p / TILE_PARTICLES), __popc(m));
        if (bs) atomicAdd(nbounce, (unsigned long long)bs);
    }
}

/* every particle left after the compaction has used its time */
__global__ void k_ch4_settle(const int64_t *d_count, int64_t *d_settled) { d_settled[0] = d_count[0]; }

void launch_advance_ch4(World &w, Species &s, double dt, const double *d_pdt, const double *d_u, int64_t nu,
                        const int64_t *d_off) {
    cudaMemsetAsync(s.ch4_bounces, 0, sizeof(unsigned long long), w.stream);
    const int64_t n = s.host_bound;
    if (n > 0) {
        Ch4Geo G;
        for (int d = 0; d < 3; d++) {
            G.x0[d] = w.g.x0[d];
            G.xm[d] = w.g.xm[d];
            G.sph[d] = w.sphere[d];
        }
        G.sph[3] = w.has_sphere ? w.sphere[3] : -1.0;
        /* one stream per (species, call) */
        const uint64_t stream = (0xC4ull << 56) | ((uint64_t)(s.id & 0xff) << 48) |
                                (s.ch4_calls & 0xffffffffffffull);
        k_advance_ch4<<<blocks_for(n, 256), 256, 0, w.stream>>>(G, s.mass, dt, s.P, s.cap, s.d_count, s.ch4_settled,
                                                                 d_pdt, d_u, nu, d_off, w.seed, stream, s.deadmask,
                                                                 s.tiledead, s.ch4_bounces, w.d_err);
        w.nlaunch++;
        launch_compact(w, s);
    }
    k_ch4_settle<<<1, 1, 0, w.stream>>>(s.d_count, s.ch4_settled);
    w.nlaunch++;
    s.ch4_calls++;
}

}  // namespace espic

namespace espic {

/* ------------------------------------------------------------------------ */
/* ch4 ion push: Species::advance(neutrals, spherium) of a charged species
 * (ch4/Species.cpp:8-91).  Pass 1, one thread per ion: the E kick over the
 * ion's whole time left (v += E (t q / m)), one move (ch4_ion_move); an ion
 * leaving the domain is dead; one striking the sphere is dead and draws its
 * neutral count (int)(mpw0 / neutral mpw0 + U(0)) and its sputter count
 * (int)(yield mpw0 / spherium mpw0 + U(1 + 11 n0)), yield 0.1 above
 * 5000 m/s.  The strike point replaces the ion's position and its speed its
 * vx (pass 2 reads them before the compaction).  cnt0 / cnt1 receive the
 * particles each ion adds to each target (0 when the strike point is
 * outside [x0, xm), which addParticle rejects, ch4/Species.cpp:103-119);
 * when both targets are one species cnt0 holds both.  Threads n .. nb write
 * the zeros that close the scans. */
struct Ch4IonArgs {
    Geo g;
    Ch4Geo G;
    double charge, mass, mpw0, dt;
    double ratio0;   /* mpw0 / neutral mpw0 */
    double sph_mpw0; /* spherium mpw0 */
    double tq[2], tm[2], tw[2]; /* target charge, mass, mpw0 */
    int same;        /* both targets are one species */
    int write_w[2];  /* the target keeps a weight row */
};

__global__ void __launch_bounds__(256) k_ch4_ion_push(Ch4IonArgs a, const double *__restrict__ ef, double *P,
                                                      int64_t stride, int64_t nb, const int64_t *__restrict__ d_count,
                                                      const int64_t *__restrict__ d_settled,
                                                      const double *__restrict__ pdt, const double *__restrict__ u,
                                                      int64_t nu, const int64_t *__restrict__ p_off, uint64_t seed,
                                                      uint64_t stream, int32_t *cnt0, int32_t *cnt1,
                                                      uint32_t *deadmask, int32_t *tiledead,
                                                      unsigned long long *nstrike, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n = d_count[0];
    bool dead = false, struck = false;
    int32_t c0 = 0, c1 = 0;
    if (p < n) {
        double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
        double v[3] = {P[3 * stride + p], P[4 * stride + p], P[5 * stride + p]};
        const double t = (pdt ? pdt[p] : (p >= d_settled[0] ? a.dt : 0.0)) + a.dt;
        double lc[3], e[3];
        xtol(a.g, x, lc);
        gather3(a.g, ef, lc, e);
        const double s = t * a.charge / a.mass;
        for (int d = 0; d < 3; d++) v[d] += e[d] * s;
        double v_mag1 = 0;
        const int res = ch4_ion_move(a.G, t, x, v, v_mag1);
        if (!(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]))) {
            atomicOr(err, DERR_NONFINITE);
            dead = true;
        } else if (res == 2) {
            dead = struck = true;
            Ch4Uniforms U{u, nu, u ? p_off[p] : 0, seed, stream, (uint64_t)p << 20, false};
            const int n0 = (int)(a.ratio0 + U(0));
            const double sput_yield = (v_mag1 > 5000) ? 0.1 : 0;
            const int n1 = (int)(sput_yield * a.mpw0 / a.sph_mpw0 + U(1 + 11 * n0));
            if (U.bad) atomicOr(err, DERR_NEUTRAL);
            if (in_bounds(a.g, x)) {
                c0 = a.same ? n0 + n1 : n0;
                c1 = a.same ? 0 : n1;
            }
            v[0] = v_mag1;
        } else {
            dead = res != 0;
        }
        for (int d = 0; d < 3; d++) {
            P[d * stride + p] = x[d];
            P[(3 + d) * stride + p] = v[d];
        }
    }
    if (p <= nb) {
        cnt0[p] = c0;
        if (cnt1) cnt1[p] = c1;
    }
    const unsigned m = __ballot_sync(0xffffffffu, dead);
    const unsigned ms = __ballot_sync(0xffffffffu, struck);
    if ((threadIdx.x & 31) == 0 && p < n) {
        deadmask[p >> 5] = m;
        if (m) atomicAdd(tiledead + (p / TILE_PARTICLES), __popc(m));
        if (ms) atomicAdd(nstrike, (unsigned long long)__popc(ms));
    }
}

/* The scanned counts' total (entry nb) grows the target: the count before
 * goes to d_count[1], the new count (at most the capacity) to d_count[0]. */
__global__ void k_ch4_ion_reserve(const int32_t *__restrict__ pre, int64_t nb, int64_t *d_count, int64_t cap,
                                  int *err) {
    const int64_t n_old = d_count[0];
    int64_t n_new = n_old + pre[nb];
    if (n_new > cap) {
        atomicOr(err, DERR_CAPACITY);
        n_new = cap;
    }
    d_count[1] = n_old;
    d_count[0] = n_new;
}

struct Ch4Target {
    double *P;
    int64_t stride, cap;
    const int64_t *d_count;
};

__device__ inline void ch4_ion_put(const Ch4IonArgs &a, const Ch4Target &T, int kind, int64_t dst, const double x[3],
                                   const double vel[3], const double e2[3]) {
    if (dst >= T.cap) return;
    for (int i = 0; i < 3; i++) {
        T.P[i * T.stride + dst] = x[i];
        T.P[(3 + i) * T.stride + dst] = vel[i] - a.tq[kind] / a.tm[kind] * e2[i] * (0.5 * a.dt);
    }
    if (a.write_w[kind]) T.P[6 * T.stride + dst] = a.tw[kind];
}

/* Pass 2, one thread per ion: a struck ion's particles in the reference's
 * order (its neutrals, then its sputtered particles), each with a diffusely
 * reflected velocity (the ion's mass in sampleVth) rewound by the target's
 * q/m E dt/2 at the strike point; ion p's particles go to its target at
 * the count before the call plus the exclusive prefix of the counts, so each
 * target receives them in ion order, as the reference's emplace_back. */
__global__ void __launch_bounds__(256) k_ch4_ion_create(Ch4IonArgs a, const double *__restrict__ ef,
                                                        const double *__restrict__ P, int64_t stride, int64_t nb,
                                                        const int32_t *__restrict__ pre0,
                                                        const int32_t *__restrict__ pre1, Ch4Target T0, Ch4Target T1,
                                                        const double *__restrict__ u, int64_t nu,
                                                        const int64_t *__restrict__ p_off, uint64_t seed,
                                                        uint64_t stream, int *err) {
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= nb) return;
    const int32_t b0 = pre0[p], c0 = pre0[p + 1] - b0;
    const int32_t b1 = a.same ? 0 : pre1[p], c1 = a.same ? 0 : pre1[p + 1] - b1;
    if (c0 + c1 == 0) return;
    const double x[3] = {P[p], P[stride + p], P[2 * stride + p]};
    const double v_mag1 = P[3 * stride + p];
    Ch4Uniforms U{u, nu, u ? p_off[p] : 0, seed, stream, (uint64_t)p << 20, false};
    const int n0 = (int)(a.ratio0 + U(0));
    const int n1 = a.same ? c0 - n0 : c1;
    double lc[3], e2[3];
    xtol(a.g, x, lc);
    gather3(a.g, ef, lc, e2);
    const int64_t base0 = T0.d_count[1] + b0;
    for (int c = 0; c < n0; c++) {
        double vel[3];
        c4_reflect(a.G, a.mass, x, v_mag1, U, 1 + 11 * c, vel);
        ch4_ion_put(a, T0, 0, base0 + c, x, vel, e2);
    }
    const Ch4Target &Ts = a.same ? T0 : T1;
    const int64_t base1 = a.same ? base0 + n0 : T1.d_count[1] + b1;
    for (int c = 0; c < n1; c++) {
        double vel[3];
        c4_reflect(a.G, a.mass, x, v_mag1, U, 2 + 11 * n0 + 11 * c, vel);
        ch4_ion_put(a, Ts, 1, base1 + c, x, vel, e2);
    }
    if (U.bad) atomicOr(err, DERR_NEUTRAL);
}

static Ch4Geo ch4_geo(const World &w) {
    Ch4Geo G;
    for (int d = 0; d < 3; d++) {
        G.x0[d] = w.g.x0[d];
        G.xm[d] = w.g.xm[d];
        G.sph[d] = w.sphere[d];
    }
    G.sph[3] = w.has_sphere ? w.sphere[3] : -1.0;
    return G;
}

void launch_advance_ch4_ions(World &w, Species &s, Species &neu, Species &sph, double dt, const double *d_pdt,
                             const double *d_u, int64_t nu, const int64_t *d_off) {
    ensure_ef64(w);
    cudaMemsetAsync(s.ch4_bounces, 0, sizeof(unsigned long long), w.stream);
    const int64_t nb = s.host_bound;
    if (nb > 0) {
        Ch4IonArgs a;
        a.g = w.g;
        a.G = ch4_geo(w);
        a.charge = s.charge;
        a.mass = s.mass;
        a.mpw0 = s.mpw0;
        a.dt = dt;
        a.ratio0 = s.mpw0 / neu.mpw0;
        a.sph_mpw0 = sph.mpw0;
        a.tq[0] = neu.charge;
        a.tm[0] = neu.mass;
        a.tw[0] = neu.mpw0;
        a.tq[1] = sph.charge;
        a.tm[1] = sph.mass;
        a.tw[1] = sph.mpw0;
        a.same = &neu == &sph;
        a.write_w[0] = !neu.uniform_w;
        a.write_w[1] = !sph.uniform_w;
        const uint64_t stream = (0xC5ull << 56) | ((uint64_t)(s.id & 0xff) << 48) |
                                (s.ch4_calls & 0xffffffffffffull);
        int32_t *cnt0 = s.ch4_cnt, *cnt1 = a.same ? nullptr : s.ch4_cnt + (nb + 1);
        int32_t *bsum = s.ch4_cnt + 2 * (nb + 1);
        k_ch4_ion_push<<<blocks_for(nb + 1, 256), 256, 0, w.stream>>>(
            a, w.ef, s.P, s.cap, nb, s.d_count, s.ch4_settled, d_pdt, d_u, nu, d_off, w.seed, stream, cnt0, cnt1,
            s.deadmask, s.tiledead, s.ch4_bounces, w.d_err);
        launch_int_excl_scan(w.stream, cnt0, nb + 1, bsum);
        k_ch4_ion_reserve<<<1, 1, 0, w.stream>>>(cnt0, nb, neu.d_count, neu.cap, w.d_err);
        if (cnt1) {
            launch_int_excl_scan(w.stream, cnt1, nb + 1, bsum);
            k_ch4_ion_reserve<<<1, 1, 0, w.stream>>>(cnt1, nb, sph.d_count, sph.cap, w.d_err);
        }
        Ch4Target T0{neu.P, neu.cap, neu.cap, neu.d_count}, T1{sph.P, sph.cap, sph.cap, sph.d_count};
        k_ch4_ion_create<<<blocks_for(nb, 256), 256, 0, w.stream>>>(a, w.ef, s.P, s.cap, nb, cnt0, cnt1, T0, T1, d_u,
                                                                     nu, d_off, w.seed, stream, w.d_err);
        w.nlaunch += 4 + (cnt1 ? 4 : 0) + 3;
        launch_compact(w, s);
    }
    k_ch4_settle<<<1, 1, 0, w.stream>>>(s.d_count, s.ch4_settled);
    w.nlaunch++;
    s.ch4_calls++;
}

/* ------------------------------------------------------------------------ */
/* ChemistryIonize::apply (ch4/Collisions.cpp:10-31), one thread per cell
 * c = (i (nj-1) + j) (nk-1) + k, the reference's loop order: n_a and
 * n_e = rho / QE gathered at the cell centre (Field_::gather's 8 terms in its
 * corner order), dni = rate n_a n_e dt, and (int)(dni dV / mpw0 + U) ions
 * (none when that is below 1 or not a number).  Uniform: u[cell_off[c]] when
 * replaying, else index c of the call's counter-based stream (the three the
 * reference draws per ion only feed World::pos(int, int, int), which
 * truncates them away, ch4/World.h:107-111).  Entry ncells .. closes the
 * scan with 0. */
__device__ __forceinline__ double gather1(const Geo &g, const double *__restrict__ f, const double lc[3]) {
    const int i = clamp_cell((int)lc[0], g.ni), j = clamp_cell((int)lc[1], g.nj), k = clamp_cell((int)lc[2], g.nk);
    const double di = lc[0] - i, dj = lc[1] - j, dk = lc[2] - k;
    const int64_t n0 = node_of(g, i, j, k), sy = g.ni, sz = (int64_t)g.ni * g.nj;
    return f[n0] * (1 - di) * (1 - dj) * (1 - dk) + f[n0 + 1] * (di) * (1 - dj) * (1 - dk) +
           f[n0 + 1 + sy] * (di) * (dj) * (1 - dk) + f[n0 + sy] * (1 - di) * (dj) * (1 - dk) +
           f[n0 + sz] * (1 - di) * (1 - dj) * (dk) + f[n0 + 1 + sz] * (di) * (1 - dj) * (dk) +
           f[n0 + 1 + sy + sz] * (di) * (dj) * (dk) + f[n0 + sy + sz] * (1 - di) * (dj) * (dk);
}

__device__ __forceinline__ void cell_ijk(const Geo &g, int64_t c, int &i, int &j, int &k) {
    const int64_t ck = g.nk - 1, cj = g.nj - 1;
    k = (int)(c % ck);
    const int64_t r = c / ck;
    j = (int)(r % cj);
    i = (int)(r / cj);
}

__global__ void __launch_bounds__(256) k_ionize_count(Geo g, const double *__restrict__ den_n,
                                                      const double *__restrict__ rho, double rate, double dt,
                                                      double dV, double mpw0, int64_t ncells,
                                                      const double *__restrict__ u, int64_t nu,
                                                      const int64_t *__restrict__ cell_off, uint64_t seed,
                                                      uint64_t stream, int32_t *cnt, int *err) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > ncells) return;
    int32_t num = 0;
    if (c < ncells) {
        int i, j, k;
        cell_ijk(g, c, i, j, k);
        const double lc[3] = {i + 0.5, j + 0.5, k + 0.5};
        const double na = gather1(g, den_n, lc);
        const double ne = gather1(g, rho, lc) / QE;
        const double dni = rate * na * ne * dt;
        double U;
        if (u) {
            const int64_t o = cell_off[c];
            if (o < 0 || o >= nu) {
                atomicOr(err, DERR_NEUTRAL);
                U = 0.0;
            } else {
                U = u[o];
            }
        } else {
            U = philox_uniform(seed, stream, (uint64_t)c);
        }
        const double y = dni * dV / mpw0 + U;
        if (y >= 2147483647.0) {
            atomicOr(err, DERR_CAPACITY);
        } else if (y >= 1) {
            num = (int32_t)y;
        }
    }
    cnt[c] = num;
}

/* Each new ion of cell (i, j, k) sits at node (i, j, k) (World::pos of the
 * truncated coordinates) with velocity 0 rewound by q/m E dt/2 (dt: the
 * world's time step, as addParticle) and weight mpw0, written after the
 * species' particles in cell order. */
__global__ void __launch_bounds__(256) k_ionize_create(Geo g, const double *__restrict__ ef, double qm,
                                                       double dt, double mpw0, int write_w, int64_t ncells,
                                                       const int32_t *__restrict__ pre, double *P, int64_t stride,
                                                       int64_t cap, const int64_t *__restrict__ d_count) {
    const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    const int32_t b = pre[c], num = pre[c + 1] - b;
    if (num <= 0) return;
    int i, j, k;
    cell_ijk(g, c, i, j, k);
    const double x[3] = {g.x0[0] + g.dh[0] * (double)i, g.x0[1] + g.dh[1] * (double)j,
                         g.x0[2] + g.dh[2] * (double)k};
    double lc[3], e[3];
    xtol(g, x, lc);
    gather3(g, ef, lc, e);
    double v[3];
    for (int d = 0; d < 3; d++) v[d] = 0.0 - qm * e[d] * (0.5 * dt);
    const int64_t base = d_count[1] + b;
    for (int q = 0; q < num; q++) {
        const int64_t dst = base + q;
        if (dst >= cap) return;
        for (int d = 0; d < 3; d++) {
            P[d * stride + dst] = x[d];
            P[(3 + d) * stride + dst] = v[d];
        }
        if (write_w) P[6 * stride + dst] = mpw0;
    }
}

void launch_ionize(World &w, const Species &neu, Species &ion, double rate, double dt, const double *d_u,
                   int64_t nu, const int64_t *d_off, int32_t *cnt, uint64_t stream) {
    const int64_t ncells = (int64_t)(w.g.ni - 1) * (w.g.nj - 1) * (w.g.nk - 1);
    const double dV = w.g.dh[0] * w.g.dh[1] * w.g.dh[2];
    int32_t *bsum = cnt + ncells + 1;
    ensure_ef64(w);
    k_ionize_count<<<blocks_for(ncells + 1, 256), 256, 0, w.stream>>>(w.g, neu.den, w.rho, rate, dt, dV, ion.mpw0,
                                                                       ncells, d_u, nu, d_off, w.seed, stream, cnt,
                                                                       w.d_err);
    launch_int_excl_scan(w.stream, cnt, ncells + 1, bsum);
    k_ch4_ion_reserve<<<1, 1, 0, w.stream>>>(cnt, ncells, ion.d_count, ion.cap, w.d_err);
    k_ionize_create<<<blocks_for(ncells, 256), 256, 0, w.stream>>>(w.g, w.ef, ion.charge / ion.mass, w.dt, ion.mpw0,
                                                                    !ion.uniform_w, ncells, cnt, ion.P, ion.cap,
                                                                    ion.cap, ion.d_count);
    w.nlaunch += 6;
}

}  // namespace espic
