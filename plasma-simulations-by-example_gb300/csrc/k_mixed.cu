/*
 * k_mixed.cu -- the mixed-precision form of the particle step: a particle is
 * an int32 cell key (i | j<<10 | k<<20), an f32 in-cell offset and an f32
 * velocity (28 bytes), with the species weight mpw0.  The push gathers E from
 * the f32 copy ef4 (one 16-byte load per corner), moves the particle in cell
 * units, applies the walls / sphere, and deposits its CIC weights as 23-bit
 * fixed-point fractions of mpw0.  The push kernel accumulates a thread
 * block's deposits in a shared-memory box spanning the block's cells (the
 * particles of a block are neighbours after the counting sort, and the common
 * drift keeps them together between sorts) with 32-bit shared atomics, then
 * adds the box to the int64 grid with one global atomic per touched node;
 * blocks whose cells span too large a box use global atomics directly.
 * Integer sums make the density independent of particle order.
 *
 * Reference behaviour restated: Species::advance (ch3/ver2/Species.cpp:7-48,
 * ch2/Species.cpp:7-38), Field_::gather/scatter (ch2/Field.h:164-208),
 * Species::computeNumberDensity (ch2/Species.cpp:41-52).  The counting sort
 * by cell has no reference counterpart (the reference never reorders
 * particles except by its removal step).
 */
#include "espic_world.h"

namespace espic {

enum { M_REFLECT = 0, M_ABSORB = 1 };

/* a corner weight in [0,1] becomes round(w * 2^23) counts of mpw0 * 2^-23;
 * 256 particles of a block cannot overflow a 32-bit shared counter */
#define MIX_Q 8388608.f
constexpr int BOX_CAP = 4096; /* nodes of the shared deposit box (16 KB) */

struct MixArgs {
    int ni, nj, nk;
    float qmdt;        /* q/m dt */
    float dtdh[3];     /* dt/dh per axis: m/s -> cells per step */
    float dh[3];
    float sx[3];       /* x0 - sphere centre */
    float r2;          /* sphere radius^2, < 0 when there is no sphere */
};

__device__ __forceinline__ void unpack(int32_t key, int &i, int &j, int &k) {
    i = key & 1023;
    j = (key >> 10) & 1023;
    k = key >> 20;
}

/* move a coordinate by v*dtdh cells (one fused multiply-add): returns the
 * new cell index, f stays in [0,1) */
__device__ __forceinline__ int advance_axis(int i, float &f, float v, float dtdh) {
    f = __fmaf_rn(v, dtdh, f);
    float fl = floorf(f);
    i += (int)fl;
    f -= fl;
    if (f >= 1.f) {
        f -= 1.f;
        i += 1;
    }
    return i;
}

__device__ __forceinline__ void reflect_axis(int &i, float &f, float &v, int n) {
    float p = (float)i + f;
    float top = (float)(n - 1);
    if (p < 0.f) {
        p = -p;
        v = -v;
    } else if (p >= top) {
        p = 2.f * top - p;
        v = -v;
    }
    int ii = (int)p;
    if (ii > n - 2) ii = n - 2;
    if (ii < 0) ii = 0;
    i = ii;
    f = p - (float)ii;
}

/* Block-wide deposit through a shared-memory box (called by every thread of
 * the block; `me` marks the threads with a particle to deposit). */
__device__ __forceinline__ void deposit_block(bool me, int32_t key, int ni, int nj, float fx, float fy, float fz,
                                              unsigned long long *acc) {
    __shared__ unsigned int sbox[BOX_CAP];
    __shared__ int s_lo[3], s_hi[3];
    int i = 0, j = 0, k = 0;
    if (me) unpack(key, i, j, k);
    if (threadIdx.x < 3) {
        s_lo[threadIdx.x] = 0x7fffffff;
        s_hi[threadIdx.x] = -1;
    }
    __syncthreads();
    int mi = __reduce_min_sync(0xffffffffu, me ? i : 0x7fffffff);
    int mj = __reduce_min_sync(0xffffffffu, me ? j : 0x7fffffff);
    int mk = __reduce_min_sync(0xffffffffu, me ? k : 0x7fffffff);
    int xi = __reduce_max_sync(0xffffffffu, me ? i : -1);
    int xj = __reduce_max_sync(0xffffffffu, me ? j : -1);
    int xk = __reduce_max_sync(0xffffffffu, me ? k : -1);
    if ((threadIdx.x & 31) == 0 && xi >= 0) {
        atomicMin(&s_lo[0], mi);
        atomicMin(&s_lo[1], mj);
        atomicMin(&s_lo[2], mk);
        atomicMax(&s_hi[0], xi);
        atomicMax(&s_hi[1], xj);
        atomicMax(&s_hi[2], xk);
    }
    __syncthreads();
    const int li = s_lo[0], lj = s_lo[1], lk = s_lo[2];
    if (s_hi[0] < 0) return; /* nothing to deposit in this block (uniform) */
    const int bi = s_hi[0] - li + 2, bj = s_hi[1] - lj + 2, bk = s_hi[2] - lk + 2;
    const int64_t vol = (int64_t)bi * bj * bk;
    float w[8];
    cic_w(fx, fy, fz, w);
    if (vol <= BOX_CAP) {
        for (int t = threadIdx.x; t < (int)vol; t += blockDim.x) sbox[t] = 0u;
        __syncthreads();
        if (me) {
            int L = ((k - lk) * bj + (j - lj)) * bi + (i - li);
            int idx[8] = {L, L + 1, L + 1 + bi, L + bi, L + bi * bj, L + 1 + bi * bj, L + 1 + bi + bi * bj,
                          L + bi + bi * bj};
#pragma unroll
            for (int c = 0; c < 8; c++) {
                unsigned q = __float2uint_rn(w[c] * MIX_Q);
                if (q) atomicAdd(&sbox[idx[c]], q);
            }
        }
        __syncthreads();
        const int64_t sy = ni, sz = (int64_t)ni * nj;
        for (int t = threadIdx.x; t < (int)vol; t += blockDim.x) {
            unsigned v = sbox[t];
            if (!v) continue;
            int ti = t % bi, r = t / bi, tj = r % bj, tk = r / bj;
            int64_t n = (int64_t)(lk + tk) * sz + (int64_t)(lj + tj) * sy + (li + ti);
            atomicAdd(acc + n, (unsigned long long)v);
        }
    } else if (me) {
        const int64_t sy = ni, sz = (int64_t)ni * nj;
        int64_t n0 = (int64_t)k * sz + (int64_t)j * sy + i;
        int64_t idx[8] = {n0, n0 + 1, n0 + 1 + sy, n0 + sy, n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
#pragma unroll
        for (int c = 0; c < 8; c++) {
            unsigned q = __float2uint_rn(w[c] * MIX_Q);
            if (q) atomicAdd(acc + idx[c], (unsigned long long)q);
        }
    }
}

/* The move of one particle once E at its position is known: v += (q/m) E dt,
 * move in cell units, then the walls (REFLECT: one mirror bounce per axis;
 * ABSORB: out of the domain or inside the sphere).  A non-finite state is
 * flagged and the particle killed.  Returns true when the particle is dead;
 * key receives the new cell. */
template <int WALLS>
__device__ __forceinline__ bool move_particle_mixed(const MixArgs &a, const float3 E, int i, int j, int k,
                                                    int32_t &key, float &fx, float &fy, float &fz, float &vx,
                                                    float &vy, float &vz, int *err) {
    vx = __fmaf_rn(E.x, a.qmdt, vx);
    vy = __fmaf_rn(E.y, a.qmdt, vy);
    vz = __fmaf_rn(E.z, a.qmdt, vz);
    i = advance_axis(i, fx, vx, a.dtdh[0]);
    j = advance_axis(j, fy, vy, a.dtdh[1]);
    k = advance_axis(k, fz, vz, a.dtdh[2]);
    bool dead = false;
    if (WALLS == M_REFLECT) {
        reflect_axis(i, fx, vx, a.ni);
        reflect_axis(j, fy, vy, a.nj);
        reflect_axis(k, fz, vz, a.nk);
    } else {
        dead = i < 0 || i > a.ni - 2 || j < 0 || j > a.nj - 2 || k < 0 || k > a.nk - 2;
        if (!dead && a.r2 >= 0.f) {
            const float rx = __fmaf_rn((float)i + fx, a.dh[0], a.sx[0]);
            const float ry = __fmaf_rn((float)j + fy, a.dh[1], a.sx[1]);
            const float rz = __fmaf_rn((float)k + fz, a.dh[2], a.sx[2]);
            dead = __fmaf_rn(rz, rz, __fmaf_rn(ry, ry, __fmul_rn(rx, rx))) <= a.r2;
        }
    }
    if (!(isfinite(fx) && isfinite(fy) && isfinite(fz) && isfinite(vx) && isfinite(vy) && isfinite(vz))) {
        atomicOr(err, DERR_NONFINITE);
        dead = true;
        i = j = k = 0;
        fx = fy = fz = 0.f;
    }
    key = (i & 1023) | ((j & 1023) << 10) | (k << 20);
    return dead;
}

/* One particle of Species::advance in the mixed form: gather E at the cell
 * corners from ef4 (one 16-byte load per corner), then the move. */
template <int WALLS>
__device__ __forceinline__ bool push_particle_mixed(const MixArgs &a, const float4 *__restrict__ ef4, int32_t &key,
                                                    float &fx, float &fy, float &fz, float &vx, float &vy,
                                                    float &vz, int *err) {
    int i, j, k;
    unpack(key, i, j, k);
    int64_t sy = a.ni, sz = (int64_t)a.ni * a.nj;
    int64_t n0 = ((int64_t)k * a.nj + j) * a.ni + i;
    float w[8];
    cic_w(fx, fy, fz, w);
    const float4 e[8] = {__ldg(ef4 + n0),      __ldg(ef4 + n0 + 1),      __ldg(ef4 + n0 + 1 + sy),      __ldg(ef4 + n0 + sy),
                         __ldg(ef4 + n0 + sz), __ldg(ef4 + n0 + 1 + sz), __ldg(ef4 + n0 + 1 + sy + sz), __ldg(ef4 + n0 + sy + sz)};
    const float3 E = gather_corners(w, e);
    return move_particle_mixed<WALLS>(a, E, i, j, k, key, fx, fy, fz, vx, vy, vz, err);
}

template <int WALLS, bool DEPOSIT>
__global__ void __launch_bounds__(256, 5) k_push_mixed(MixArgs a, const float4 *__restrict__ ef4, int32_t *cell,
                                                    float *off, float *vel, int64_t stride,
                                                    const int64_t *__restrict__ d_count, uint32_t *deadmask,
                                                    int32_t *tiledead, unsigned long long *acc, int *err) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t n = d_count[0];
    bool live = p < n;
    bool dead = false;
    int32_t key = -1;
    float fx = 0, fy = 0, fz = 0;
    if (live) {
        key = cell[p];
        fx = off[p];
        fy = off[stride + p];
        fz = off[2 * stride + p];
        float vx = vel[p], vy = vel[stride + p], vz = vel[2 * stride + p];
        dead = push_particle_mixed<WALLS>(a, ef4, key, fx, fy, fz, vx, vy, vz, err);
        cell[p] = key;
        off[p] = fx;
        off[stride + p] = fy;
        off[2 * stride + p] = fz;
        vel[p] = vx;
        vel[stride + p] = vy;
        vel[2 * stride + p] = vz;
    }
    if (DEPOSIT) deposit_block(live && !dead, key, a.ni, a.nj, fx, fy, fz, acc);
    if (WALLS == M_ABSORB) {
        unsigned m = __ballot_sync(0xffffffffu, dead);
        if ((threadIdx.x & 31) == 0 && live) {
            deadmask[p >> 5] = m;
            if (m) atomicAdd(tiledead + (p / TILE_PARTICLES), __popc(m));
        }
    }
}

/* ---------------------------------------------------------------------- */
/* The push over tile segments.  After a counting sort the particles lie in
 * tile-major cell order (tiles of TILE_CELLS^3 cells, cells row-major within
 * a tile), and seg[t] is the first particle of tile t.  One thread block
 * takes one tile's segment: it stages the float E of a TBW^3-node box
 * around the segment's particles in shared memory, pushes the particles
 * 256 at a time with the E gather read from that box, and deposits their
 * 2^-23 fixed-point corner weights into a shared TBW^3-node integer box,
 * which it adds to the grid once at the end (one global atomic per touched
 * node).  The box is centred on the per-axis median cell of 32 keys spread
 * over the segment, so it follows the drift of the segment's particles
 * between sorts; particles outside it (the few that moved more than three
 * cells from their tile, and particles the removal moved into the segment)
 * gather from global memory and deposit with global atomics.  The arithmetic
 * per particle is push_particle_mixed's; the integer sums do not depend on
 * where they are accumulated, so the charge equals that of k_push_mixed bit
 * for bit.  Particles appended since the sort (after seg[ntiles]) are pushed
 * by k_push_tail. */
/* nodes per edge of a block's E and deposit box: 13 (11 cells, a tile and
 * 1.5 cells on each side) at 44 KB of shared memory and 64 registers fits
 * four blocks per SM; measured at 14.6 ions per cell over the 20 steps
 * between sorts, 7% faster than 15 at three blocks per SM */
constexpr int TBW = 13;

/* The block's sums of four per-thread floats as float64 (warp butterflies
 * in float, then the warps in order), written by thread 0..3.  Every thread
 * of the block calls it. */
__device__ __forceinline__ void block_dsum(float f1, float f2, float f3, float f4, double *out) {
    __shared__ double wsum[8][4];
    float v[4] = {f1, f2, f3, f4};
#pragma unroll
    for (int q = 0; q < 4; q++)
        for (int o = 16; o > 0; o >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], o);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 4; q++) wsum[threadIdx.x >> 5][q] = (double)v[q];
    __syncthreads();
    if (threadIdx.x < 4) {
        double t = 0;
        for (int w8 = 0; w8 < (int)(blockDim.x >> 5); w8++) t += wsum[w8][threadIdx.x];
        out[threadIdx.x] = t;
    }
}

/* the median over the warp of one int per lane (the 16th smallest) */
__device__ __forceinline__ int warp_median(int v) {
    int below = 0, same = 0;
#pragma unroll 8
    for (int l = 0; l < 32; l++) {
        const int x = __shfl_sync(0xffffffffu, v, l);
        below += x < v;
        same += x == v;
    }
    const unsigned pick = __ballot_sync(0xffffffffu, below <= 15 && below + same > 15);
    return __shfl_sync(0xffffffffu, v, __ffs(pick) - 1);
}

template <int WALLS, bool DEPOSIT>
__global__ void __launch_bounds__(256, 4) k_push_tiles(MixArgs a, const float4 *__restrict__ ef4, int32_t *cell,
                                                    float *off, float *vel, int64_t stride,
                                                    const int32_t *__restrict__ seg,
                                                    const int64_t *__restrict__ d_count, uint32_t *deadmask,
                                                    int32_t *tiledead, unsigned long long *acc, int *err,
                                                    double *dsum) {
    constexpr int BV = TBW * TBW * TBW;
    extern __shared__ __align__(16) unsigned char tile_smem[];
    float4 *sE = (float4 *)tile_smem;
    unsigned int *sD = (unsigned int *)(tile_smem + BV * sizeof(float4));
    __shared__ int s_lo[3];
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int64_t n = d_count[0];
    const int p0 = seg[blockIdx.x];
    const int p1 = (int)min((int64_t)seg[blockIdx.x + 1], n);
    if (p1 <= p0) { /* block-uniform */
        if (dsum && threadIdx.x < 4) dsum[4 * (int64_t)blockIdx.x + threadIdx.x] = 0.0;
        return;
    }
    if (warp == 0) {
        const int q = p0 + (int)(((int64_t)(p1 - p0) * lane) >> 5);
        int i, j, k;
        unpack(cell[q], i, j, k);
        const int c[3] = {warp_median(i), warp_median(j), warp_median(k)};
        const int ncell[3] = {a.ni - 1, a.nj - 1, a.nk - 1};
        if (lane < 3) {
            int lo = c[lane] - (TBW - 1) / 2;
            if (lo > ncell[lane] - (TBW - 1)) lo = ncell[lane] - (TBW - 1);
            if (lo < 0) lo = 0;
            s_lo[lane] = lo; /* box nodes lo .. lo + TBW - 1, cells lo .. lo + TBW - 2 */
        }
    }
    if (DEPOSIT)
        for (int t = threadIdx.x; t < BV; t += blockDim.x) sD[t] = 0u;
    __syncthreads();
    const int li = s_lo[0], lj = s_lo[1], lk = s_lo[2];
    const int sy = a.ni, sz = a.ni * a.nj;
    /* the box's 2197 nodes, nine per thread with every load issued before
     * the stores (one memory latency for the whole box, not one per row) */
    {
        constexpr int PER = (BV + 255) / 256;
        float4 ev[PER];
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int t = threadIdx.x + q * 256;
            const int tt = t < BV ? t : 0;
            const int tk = tt / (TBW * TBW), rem = tt - tk * TBW * TBW, tj = rem / TBW, ti = rem - tj * TBW;
            ev[q] = __ldg(ef4 + ((int64_t)(lk + tk) * sz + (int64_t)(lj + tj) * sy + li + ti));
        }
#pragma unroll
        for (int q = 0; q < PER; q++) {
            const int t = threadIdx.x + q * 256;
            if (t < BV) sE[t] = ev[q];
        }
    }
    __syncthreads();
    float *off1 = off + stride, *off2 = off + 2 * stride, *vel1 = vel + stride, *vel2 = vel + 2 * stride;
    /* the diagnostics' sums over the pushed particles (count, v, |v|^2) */
    float f1 = 0.f, f2 = 0.f, f3 = 0.f, f4 = 0.f;
    for (int base = p0; base < p1; base += blockDim.x) {
        const int p = base + threadIdx.x;
        const bool live = p < p1;
        bool dead = false;
        int32_t key = -1;
        float fx = 0.f, fy = 0.f, fz = 0.f;
        if (live) {
            key = cell[p];
            fx = off[p];
            fy = off1[p];
            fz = off2[p];
            float vx = vel[p], vy = vel1[p], vz = vel2[p];
            int i, j, k;
            unpack(key, i, j, k);
            float w[8];
            cic_w(fx, fy, fz, w);
            float4 e[8];
            const int bi = i - li, bj = j - lj, bk = k - lk;
            if ((unsigned)bi < TBW - 1 && (unsigned)bj < TBW - 1 && (unsigned)bk < TBW - 1) {
                const int L = (bk * TBW + bj) * TBW + bi;
                e[0] = sE[L];
                e[1] = sE[L + 1];
                e[2] = sE[L + 1 + TBW];
                e[3] = sE[L + TBW];
                e[4] = sE[L + TBW * TBW];
                e[5] = sE[L + 1 + TBW * TBW];
                e[6] = sE[L + 1 + TBW + TBW * TBW];
                e[7] = sE[L + TBW + TBW * TBW];
            } else {
                const float4 *E0 = ef4 + (((int64_t)k * a.nj + j) * a.ni + i);
                e[0] = __ldg(E0);
                e[1] = __ldg(E0 + 1);
                e[2] = __ldg(E0 + 1 + sy);
                e[3] = __ldg(E0 + sy);
                e[4] = __ldg(E0 + sz);
                e[5] = __ldg(E0 + 1 + sz);
                e[6] = __ldg(E0 + 1 + sy + sz);
                e[7] = __ldg(E0 + sy + sz);
            }
            const float3 E = gather_corners(w, e);
            dead = move_particle_mixed<WALLS>(a, E, i, j, k, key, fx, fy, fz, vx, vy, vz, err);
            cell[p] = key;
            off[p] = fx;
            off1[p] = fy;
            off2[p] = fz;
            vel[p] = vx;
            vel1[p] = vy;
            vel2[p] = vz;
            if (!dead) {
                f1 += vx;
                f2 += vy;
                f3 += vz;
                f4 += vx * vx + vy * vy + vz * vz;
            }
            if (WALLS == M_ABSORB && dead) {
                atomicOr(deadmask + (p >> 5), 1u << (p & 31));
                atomicAdd(tiledead + (p / TILE_PARTICLES), 1);
            }
        }
        if (DEPOSIT && live && !dead) {
            float w[8];
            cic_w(fx, fy, fz, w);
            int i, j, k;
            unpack(key, i, j, k);
            const int bi = i - li, bj = j - lj, bk = k - lk;
            if ((unsigned)bi < TBW - 1 && (unsigned)bj < TBW - 1 && (unsigned)bk < TBW - 1) {
                const int L = (bk * TBW + bj) * TBW + bi;
                const int idx[8] = {L,           L + 1,           L + 1 + TBW,           L + TBW,
                                    L + TBW * TBW, L + 1 + TBW * TBW, L + 1 + TBW + TBW * TBW, L + TBW + TBW * TBW};
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const unsigned q = __float2uint_rn(w[c] * MIX_Q);
                    if (q) atomicAdd(&sD[idx[c]], q);
                }
            } else {
                const int64_t n0 = ((int64_t)k * a.nj + j) * a.ni + i;
                const int64_t idx[8] = {n0,      n0 + 1,      n0 + 1 + sy,      n0 + sy,
                                        n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
#pragma unroll
                for (int c = 0; c < 8; c++) {
                    const unsigned q = __float2uint_rn(w[c] * MIX_Q);
                    if (q) atomicAdd(acc + idx[c], (unsigned long long)q);
                }
            }
        }
    }
    if (dsum) block_dsum(f1, f2, f3, f4, dsum + 4 * (int64_t)blockIdx.x);
    if (!DEPOSIT) return;
    __syncthreads();
    for (int r = warp; r < TBW * TBW; r += nwarps) {
        const int tk = r / TBW, tj = r - tk * TBW;
        unsigned long long *dst = acc + ((int64_t)(lk + tk) * sz + (int64_t)(lj + tj) * sy + li);
        for (int ti = lane; ti < TBW; ti += 32) {
            const unsigned v = sD[r * TBW + ti];
            if (v) atomicAdd(dst + ti, (unsigned long long)v);
        }
    }
}

/* The deposit alone over tile segments (Species::computeNumberDensity of
 * a sorted mixed species whose push did not deposit): one block per tile
 * segment, the 2^-23 fixed-point corner weights of deposit_block summed in
 * a shared TBW^3-node box placed as k_push_tiles places it (the per-axis
 * median cell of 32 keys of the segment), ions outside the box through
 * global atomics, the box added to the grid once.  The integer sums equal
 * those of k_deposit_mixed bit for bit. */
__global__ void __launch_bounds__(256) k_deposit_tiles(MixArgs a, const int32_t *__restrict__ cell,
                                                       const float *__restrict__ off, int64_t stride,
                                                       const int32_t *__restrict__ seg,
                                                       const int64_t *__restrict__ d_count,
                                                       unsigned long long *acc) {
    constexpr int BV = TBW * TBW * TBW;
    __shared__ unsigned int sD[BV];
    __shared__ int s_lo[3];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int64_t n = d_count[0];
    const int p0 = seg[blockIdx.x];
    const int p1 = (int)min((int64_t)seg[blockIdx.x + 1], n);
    if (p1 <= p0) return; /* block-uniform */
    if (warp == 0) {
        const int q = p0 + (int)(((int64_t)(p1 - p0) * lane) >> 5);
        int i, j, k;
        unpack(cell[q], i, j, k);
        const int c[3] = {warp_median(i), warp_median(j), warp_median(k)};
        const int ncell[3] = {a.ni - 1, a.nj - 1, a.nk - 1};
        if (lane < 3) {
            int lo = c[lane] - (TBW - 1) / 2;
            if (lo > ncell[lane] - (TBW - 1)) lo = ncell[lane] - (TBW - 1);
            if (lo < 0) lo = 0;
            s_lo[lane] = lo;
        }
    }
    for (int t = threadIdx.x; t < BV; t += blockDim.x) sD[t] = 0u;
    __syncthreads();
    const int li = s_lo[0], lj = s_lo[1], lk = s_lo[2];
    const int64_t sy = a.ni, sz = (int64_t)a.ni * a.nj;
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        int i, j, k;
        unpack(cell[p], i, j, k);
        float w[8];
        cic_w(off[p], off[stride + p], off[2 * stride + p], w);
        const int bi = i - li, bj = j - lj, bk = k - lk;
        if ((unsigned)bi < TBW - 1 && (unsigned)bj < TBW - 1 && (unsigned)bk < TBW - 1) {
            const int L = (bk * TBW + bj) * TBW + bi;
            const int idx[8] = {L,           L + 1,           L + 1 + TBW,           L + TBW,
                                L + TBW * TBW, L + 1 + TBW * TBW, L + 1 + TBW + TBW * TBW, L + TBW + TBW * TBW};
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const unsigned q = __float2uint_rn(w[c] * MIX_Q);
                if (q) atomicAdd(&sD[idx[c]], q);
            }
        } else {
            const int64_t n0 = ((int64_t)k * a.nj + j) * a.ni + i;
            const int64_t idx[8] = {n0,      n0 + 1,      n0 + 1 + sy,      n0 + sy,
                                    n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const unsigned q = __float2uint_rn(w[c] * MIX_Q);
                if (q) atomicAdd(acc + idx[c], (unsigned long long)q);
            }
        }
    }
    __syncthreads();
    for (int r = warp; r < TBW * TBW; r += nwarps) {
        const int tk = r / TBW, tj = r - tk * TBW;
        unsigned long long *dst = acc + ((int64_t)(lk + tk) * sz + (int64_t)(lj + tj) * sy + li);
        for (int ti = lane; ti < TBW; ti += 32) {
            const unsigned v = sD[r * TBW + ti];
            if (v) atomicAdd(dst + ti, (unsigned long long)v);
        }
    }
}

/* the deposit alone of the particles appended since the sort: [first, n),
 * grid-stride, global atomics */
__global__ void __launch_bounds__(256) k_deposit_tail(MixArgs a, const int32_t *__restrict__ cell,
                                                      const float *__restrict__ off, int64_t stride,
                                                      const int32_t *__restrict__ first,
                                                      const int64_t *__restrict__ d_count,
                                                      unsigned long long *acc) {
    const int64_t n = d_count[0];
    const int64_t sy = a.ni, sz = (int64_t)a.ni * a.nj;
    for (int64_t p = first[0] + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        int i, j, k;
        unpack(cell[p], i, j, k);
        float w[8];
        cic_w(off[p], off[stride + p], off[2 * stride + p], w);
        const int64_t n0 = ((int64_t)k * a.nj + j) * a.ni + i;
        const int64_t idx[8] = {n0,      n0 + 1,      n0 + 1 + sy,      n0 + sy,
                                n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const unsigned q = __float2uint_rn(w[c] * MIX_Q);
            if (q) atomicAdd(acc + idx[c], (unsigned long long)q);
        }
    }
}

/* particles appended since the sort: [seg[ntiles], n), grid-stride, the
 * particle step of push_particle_mixed and global-atomic deposits */
template <int WALLS, bool DEPOSIT>
__global__ void __launch_bounds__(256) k_push_tail(MixArgs a, const float4 *__restrict__ ef4, int32_t *cell,
                                                   float *off, float *vel, int64_t stride,
                                                   const int32_t *__restrict__ first,
                                                   const int64_t *__restrict__ d_count, uint32_t *deadmask,
                                                   int32_t *tiledead, unsigned long long *acc, int *err,
                                                   double *dsum) {
    const int64_t n = d_count[0];
    const int64_t sy = a.ni, sz = (int64_t)a.ni * a.nj;
    float f1 = 0.f, f2 = 0.f, f3 = 0.f, f4 = 0.f;
    for (int64_t p = first[0] + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        int32_t key = cell[p];
        float fx = off[p], fy = off[stride + p], fz = off[2 * stride + p];
        float vx = vel[p], vy = vel[stride + p], vz = vel[2 * stride + p];
        const bool dead = push_particle_mixed<WALLS>(a, ef4, key, fx, fy, fz, vx, vy, vz, err);
        cell[p] = key;
        off[p] = fx;
        off[stride + p] = fy;
        off[2 * stride + p] = fz;
        vel[p] = vx;
        vel[stride + p] = vy;
        vel[2 * stride + p] = vz;
        if (!dead) {
            f1 += vx;
            f2 += vy;
            f3 += vz;
            f4 += vx * vx + vy * vy + vz * vz;
        }
        if (WALLS == M_ABSORB && dead) {
            atomicOr(deadmask + (p >> 5), 1u << (p & 31));
            atomicAdd(tiledead + (p / TILE_PARTICLES), 1);
        }
        if (DEPOSIT && !dead) {
            int i, j, k;
            unpack(key, i, j, k);
            float w[8];
            cic_w(fx, fy, fz, w);
            const int64_t n0 = ((int64_t)k * a.nj + j) * a.ni + i;
            const int64_t idx[8] = {n0,      n0 + 1,      n0 + 1 + sy,      n0 + sy,
                                    n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
#pragma unroll
            for (int c = 0; c < 8; c++) {
                const unsigned q = __float2uint_rn(w[c] * MIX_Q);
                if (q) atomicAdd(acc + idx[c], (unsigned long long)q);
            }
        }
    }
    if (dsum) block_dsum(f1, f2, f3, f4, dsum + 4 * (int64_t)blockIdx.x);
}

__global__ void __launch_bounds__(256) k_deposit_mixed(MixArgs a, const int32_t *__restrict__ cell,
                                                       const float *__restrict__ off, int64_t stride,
                                                       const int64_t *__restrict__ d_count,
                                                       unsigned long long *acc) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool me = p < d_count[0];
    int32_t key = -1;
    float fx = 0, fy = 0, fz = 0;
    if (me) {
        key = cell[p];
        fx = off[p];
        fy = off[stride + p];
        fz = off[2 * stride + p];
    }
    deposit_block(me, key, a.ni, a.nj, fx, fy, fz, acc);
}

/* ---------------------------------------------------------------------- */
/* Batched ensemble: push (reflecting walls, the ch2 box) and CIC deposit of
 * every box and species in one launch over a flattened work list.  Work item
 * w = (segment, first particle, count) lies inside one species of one box;
 * blocks take items w = blockIdx.x, + gridDim.x, ...  The particle arithmetic
 * is push_particle_mixed, the deposit the same 2^-23 fixed-point counts as
 * deposit_block, so a box of the ensemble evolves bit for bit like the same
 * box run as a World.  With PUSH false the items are only deposited. */
template <bool PUSH>
__global__ void __launch_bounds__(512) k_ens_push(const EnsBox *__restrict__ boxes, const EnsSeg *__restrict__ segs,
                                                  const int4 *__restrict__ work, int nwork,
                                                  const float4 *__restrict__ ef4, int32_t *cell, float *off,
                                                  float *vel, int64_t stride, unsigned long long *acc,
                                                  int64_t total_nodes, int *err) {
    for (int wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const int4 W = work[wi];
        const EnsSeg sg = segs[W.x];
        const EnsBox B = boxes[sg.box];
        MixArgs a;
        a.ni = B.g.ni;
        a.nj = B.g.nj;
        a.nk = B.g.nk;
        a.qmdt = sg.qmdt;
        for (int d = 0; d < 3; d++) {
            a.dtdh[d] = B.dtdh[d];
            a.dh[d] = (float)B.g.dh[d];
            a.sx[d] = 0.f;
        }
        a.r2 = -1.f;
        const float4 *E = ef4 + B.node0;
        unsigned long long *A = acc + (int64_t)sg.sp * total_nodes + B.node0;
        const int64_t sy = a.ni, sz = (int64_t)a.ni * a.nj;
        for (int q = threadIdx.x; q < W.z; q += blockDim.x) {
            const int64_t p = sg.p0 + W.y + q;
            int32_t key = cell[p];
            float fx = off[p], fy = off[stride + p], fz = off[2 * stride + p];
            bool dead = false;
            if (PUSH) {
                float vx = vel[p], vy = vel[stride + p], vz = vel[2 * stride + p];
                dead = push_particle_mixed<M_REFLECT>(a, E, key, fx, fy, fz, vx, vy, vz, err);
                cell[p] = key;
                off[p] = fx;
                off[stride + p] = fy;
                off[2 * stride + p] = fz;
                vel[p] = vx;
                vel[stride + p] = vy;
                vel[2 * stride + p] = vz;
            }
            if (dead) continue;
            int i, j, k;
            unpack(key, i, j, k);
            const int64_t n0 = (int64_t)k * sz + (int64_t)j * sy + i;
            const int64_t idx[8] = {n0,      n0 + 1,      n0 + 1 + sy,      n0 + sy,
                                    n0 + sz, n0 + 1 + sz, n0 + 1 + sy + sz, n0 + sy + sz};
            float w[8];
            cic_w(fx, fy, fz, w);
#pragma unroll
            for (int c = 0; c < 8; c++) {
                unsigned qc = __float2uint_rn(w[c] * MIX_Q);
                if (qc) atomicAdd(A + idx[c], (unsigned long long)qc);
            }
        }
    }
}

void launch_ens_push(cudaStream_t st, bool push, int blocks, int threads, const EnsBox *boxes, const EnsSeg *segs,
                     const int4 *work, int nwork, const float4 *ef4, int32_t *cell, float *off, float *vel,
                     int64_t stride, unsigned long long *acc, int64_t total_nodes, int *err) {
    if (nwork <= 0) return;
    if (push)
        k_ens_push<true><<<blocks, threads, 0, st>>>(boxes, segs, work, nwork, ef4, cell, off, vel, stride, acc,
                                                     total_nodes, err);
    else
        k_ens_push<false><<<blocks, threads, 0, st>>>(boxes, segs, work, nwork, ef4, cell, off, vel, stride, acc,
                                                      total_nodes, err);
}

/* mixed form -> float64 block for n particles from row `first` */
__global__ void k_from_mixed_n(Geo g, const int32_t *__restrict__ cell, const float *__restrict__ off,
                               const float *__restrict__ vel, int64_t stride, int64_t first, int64_t n, double w0,
                               double *P, int64_t pstride) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int64_t p = first + t;
    int i[3];
    unpack(cell[p], i[0], i[1], i[2]);
    for (int d = 0; d < 3; d++) {
        P[d * pstride + t] = __fma_rn((double)i[d] + (double)off[d * stride + p], g.dh[d], g.x0[d]);
        P[(3 + d) * pstride + t] = (double)vel[d * stride + p];
    }
    P[6 * pstride + t] = w0;
}

/* float64 block -> mixed form (World::XtoL in float64, then split) */
__global__ void k_to_mixed(Geo g, const double *__restrict__ P, int64_t pstride, int64_t n, int64_t first,
                           int32_t *cell, float *off, float *vel, int64_t stride) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    int64_t dst = first + t;
    int c[3];
    int nmax[3] = {g.ni, g.nj, g.nk};
    for (int d = 0; d < 3; d++) {
        double lc = (P[d * pstride + t] - g.x0[d]) / g.dh[d];
        int i = (int)lc;
        if (i < 0) i = 0;
        if (i > nmax[d] - 2) i = nmax[d] - 2;
        c[d] = i;
        off[d * stride + dst] = (float)(lc - i);
        vel[d * stride + dst] = (float)P[(3 + d) * pstride + t];
    }
    cell[dst] = c[0] | (c[1] << 10) | (c[2] << 20);
}

/* mixed form -> float64 block (x = x0 + (i + f) dh) */
__global__ void k_from_mixed(Geo g, const int32_t *__restrict__ cell, const float *__restrict__ off,
                             const float *__restrict__ vel, int64_t stride, const int64_t *__restrict__ d_count,
                             double w0, double *P, int64_t pstride) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= d_count[0]) return;
    int i[3];
    unpack(cell[p], i[0], i[1], i[2]);
    for (int d = 0; d < 3; d++) {
        P[d * pstride + p] = __fma_rn((double)i[d] + (double)off[d * stride + p], g.dh[d], g.x0[d]);
        P[(3 + d) * pstride + p] = (double)vel[d * stride + p];
    }
    P[6 * pstride + p] = w0;
}

/* ---------------------------------------------------------------------- */
/* counting sort by cell: histogram, exclusive scan, scatter               */
/* the sort order: tile-major (tiles of TILE_CELLS^3 cells, ntx x nty tiles
 * per plane of tiles), cells row-major within a tile; partial tiles at the
 * far faces leave unused slots */
__device__ __forceinline__ int32_t linear_cell(int32_t key, int ntx, int nty) {
    int i, j, k;
    unpack(key, i, j, k);
    const int tile = ((k / TILE_CELLS) * nty + (j / TILE_CELLS)) * ntx + (i / TILE_CELLS);
    return (tile * TILE_CELLS + (k % TILE_CELLS)) * TILE_CELLS * TILE_CELLS + (j % TILE_CELLS) * TILE_CELLS +
           (i % TILE_CELLS);
}

/* seg[t] = first particle of tile t (from the exclusive scan of the cell
 * counts), seg[ntiles] = the count */
__global__ void k_tile_seg(const int32_t *__restrict__ counts, int64_t ntiles, const int64_t *__restrict__ d_count,
                           int32_t *seg) {
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntiles) seg[t] = counts[t * TILE_CELLS * TILE_CELLS * TILE_CELLS];
    if (t == ntiles) seg[t] = (int32_t)d_count[0];
}

/* Runs of equal cells in lane order (the particles are nearly sorted, so a
 * warp holds a few long runs): each lane gets the first lane of its run and
 * the run length.  A cell that appears in several runs is counted once per
 * run, which leaves sums and slot ranges exact.  Every lane of the warp
 * calls it; lanes without a particle pass -1 and form runs of their own. */
__device__ __forceinline__ void cell_runs(int32_t lc, int &head, int &len) {
    const int lane = threadIdx.x & 31;
    const int32_t prev = __shfl_up_sync(0xffffffffu, lc, 1);
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || prev != lc || lc < 0);
    const unsigned le = 0xffffffffu >> (31 - lane);
    head = 31 - __clz(heads & le);
    const unsigned after = heads & ~le;
    const int next = after ? __ffs(after) - 1 : 32;
    len = next - head;
}

__global__ void __launch_bounds__(256) k_sort_hist(const int32_t *__restrict__ cell,
                                                   const int64_t *__restrict__ d_count, int ntx, int nty,
                                                   int32_t *counts) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool me = p < d_count[0];
    int32_t lc = me ? linear_cell(cell[p], ntx, nty) : -1;
    int head, len;
    cell_runs(lc, head, len);
    if (me && (int)(threadIdx.x & 31) == head) atomicAdd(counts + lc, len);
}

constexpr int SCAN_PER_BLOCK = 8192; /* 1024 threads x 8 */

__device__ __forceinline__ int32_t scan_block(int32_t v, int32_t *sh, int32_t *total) {
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

__global__ void __launch_bounds__(1024) k_scan_reduce(const int32_t *__restrict__ x, int64_t n, int32_t *bsum) {
    __shared__ int32_t sh[32];
    int64_t base = (int64_t)blockIdx.x * SCAN_PER_BLOCK + threadIdx.x * 8;
    int32_t s = 0;
#pragma unroll
    for (int q = 0; q < 8; q++)
        if (base + q < n) s += x[base + q];
    int32_t tot;
    scan_block(s, sh, &tot);
    if (threadIdx.x == 0) bsum[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(1024) k_scan_bsum(int32_t *bsum, int64_t nb) {
    __shared__ int32_t sh[32];
    int64_t per = (nb + 1023) / 1024;
    int64_t a = threadIdx.x * per, b = a + per;
    if (b > nb) b = nb;
    int32_t s = 0;
    for (int64_t i = a; i < b; i++) s += bsum[i];
    int32_t run = scan_block(s, sh, nullptr);
    for (int64_t i = a; i < b; i++) {
        int32_t c = bsum[i];
        bsum[i] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(1024) k_scan_down(int32_t *x, int64_t n, const int32_t *__restrict__ bsum) {
    __shared__ int32_t sh[32];
    int64_t base = (int64_t)blockIdx.x * SCAN_PER_BLOCK + threadIdx.x * 8;
    int32_t v[8], s = 0;
#pragma unroll
    for (int q = 0; q < 8; q++) {
        v[q] = (base + q < n) ? x[base + q] : 0;
        s += v[q];
    }
    int32_t run = scan_block(s, sh, nullptr) + bsum[blockIdx.x];
#pragma unroll
    for (int q = 0; q < 8; q++) {
        if (base + q < n) x[base + q] = run;
        run += v[q];
    }
}

/* The sort's scatter writes only each particle's index to its slot
 * (perm[dst] = p); the particle's fields are then gathered slot by slot, one
 * array per pass so that the span of source particles a stretch of slots
 * draws from stays in L2 (a slot's particles come from a few planes of
 * cells around its own, shifted by the drift).  Twenty steps after the
 * previous sort of 450M ions, writing the seven fields from the source side
 * took 71 ms, gathering all seven in one pass 22 ms, one array per pass
 * 18 ms (plus 7 ms of histogram, scan and index scatter). */
__global__ void __launch_bounds__(256) k_sort_scatter(const int32_t *__restrict__ cell,
                                                      const int64_t *__restrict__ d_count, int ntx, int nty,
                                                      int32_t *cursor, int32_t *perm) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool me = p < d_count[0];
    int32_t lc = me ? linear_cell(cell[p], ntx, nty) : -1;
    int head, len;
    cell_runs(lc, head, len);
    const int lane = threadIdx.x & 31;
    int32_t base = 0;
    if (me && lane == head) base = atomicAdd(cursor + lc, len);
    base = __shfl_sync(0xffffffffu, base, head);
    if (!me) return;
    perm[base + (lane - head)] = (int32_t)p;
}

/* The whole particle in one pass: q's source index p = perm[q] is read
 * once, then the key and the six float rows are gathered from p and written
 * at q (offsets and velocities to the second set of arrays, the key over
 * perm in place: each thread reads its slots before writing them).  An index
 * outside the species, which the histogram and scatter cannot produce, is
 * flagged, not read.  A block takes 4096 consecutive slots (four per
 * thread, one block per SM): the thermal spread sends the ions of a source
 * sector to cells a few slots apart, so a block that holds a long run of
 * slots finds most sector-mates of its sources still in the SM's L1. */
constexpr int GATHER_THREADS = 1024, GATHER_PER = 4; /* one block of 4096 slots per SM at a time */

__global__ void __launch_bounds__(GATHER_THREADS, 1) k_sort_gather_all(const int32_t *__restrict__ cell,
                                                                       const float *__restrict__ off,
                                                                       const float *__restrict__ vel, int64_t stride,
                                                                       const int64_t *__restrict__ d_count,
                                                                       int32_t *perm_key, float *off2, float *vel2,
                                                                       int *err) {
    const int64_t n = d_count[0];
    const int64_t q0 = (int64_t)blockIdx.x * (GATHER_THREADS * GATHER_PER) + threadIdx.x;
    int64_t p[GATHER_PER];
#pragma unroll
    for (int h = 0; h < GATHER_PER; h++) {
        const int64_t q = q0 + h * GATHER_THREADS;
        p[h] = q < n ? perm_key[q] : -1;
        if (q < n && (p[h] < 0 || p[h] >= n)) {
            atomicOr(err, DERR_SORT);
            p[h] = -1;
        }
    }
    int32_t key[GATHER_PER];
    float v[GATHER_PER][6];
#pragma unroll
    for (int h = 0; h < GATHER_PER; h++) {
        if (p[h] < 0) continue;
        key[h] = cell[p[h]];
#pragma unroll
        for (int d = 0; d < 3; d++) {
            v[h][d] = off[d * stride + p[h]];
            v[h][3 + d] = vel[d * stride + p[h]];
        }
    }
#pragma unroll
    for (int h = 0; h < GATHER_PER; h++) {
        if (p[h] < 0) continue;
        const int64_t q = q0 + h * GATHER_THREADS;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            off2[d * stride + q] = v[h][d];
            vel2[d * stride + q] = v[h][3 + d];
        }
        perm_key[q] = key[h];
    }
}

/* Per block: count, sum v and sum |v|^2 of a mixed species.  Each thread
 * takes four particles a pass (all twelve loads issued before the sums, so
 * the pass is bound by bandwidth, not by the loads' latency); the float sums
 * of every 32 particles are added into float64. */
__global__ void __launch_bounds__(256) k_diag_mixed(const float *__restrict__ vel, int64_t stride,
                                                    const int64_t *__restrict__ d_count, double *partials,
                                                    int nblocks) {
    const int64_t n = d_count[0];
    const int64_t S = (int64_t)nblocks * 256;
    double acc[5] = {0, 0, 0, 0, 0};
    float f[5] = {0, 0, 0, 0, 0};
    int run = 0;
    for (int64_t p0 = (int64_t)blockIdx.x * 256 + threadIdx.x; p0 < n; p0 += 4 * S) {
        float v[4][3];
        bool ok[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int64_t p = p0 + h * S;
            ok[h] = p < n;
#pragma unroll
            for (int c = 0; c < 3; c++) v[h][c] = ok[h] ? vel[c * stride + p] : 0.f;
        }
#pragma unroll
        for (int h = 0; h < 4; h++) {
            if (!ok[h]) continue;
            f[0] += 1.f;
            f[1] += v[h][0];
            f[2] += v[h][1];
            f[3] += v[h][2];
            f[4] += v[h][0] * v[h][0] + v[h][1] * v[h][1] + v[h][2] * v[h][2];
        }
        if (++run == 8) {
            for (int q = 0; q < 5; q++) {
                acc[q] += (double)f[q];
                f[q] = 0.f;
            }
            run = 0;
        }
    }
    for (int q = 0; q < 5; q++) acc[q] += (double)f[q];
    __shared__ double sh[5][8];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = 0; q < 5; q++) {
        double x = acc[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][wid] = x;
    }
    __syncthreads();
    if (threadIdx.x < 5) {
        double s = 0;
        for (int k = 0; k < 8; k++) s += sh[threadIdx.x][k];
        partials[5 * blockIdx.x + threadIdx.x] = s;
    }
}

__global__ void k_diag_mixed_final(const double *__restrict__ partials, int nblocks, double mass, double w0,
                                   double *out) {
    int lane = threadIdx.x & 31;
    double s[5] = {0, 0, 0, 0, 0};
    for (int b = lane; b < nblocks; b += 32)
        for (int q = 0; q < 5; q++) s[q] += partials[5 * b + q];
    for (int q = 0; q < 5; q++)
        for (int o = 16; o > 0; o >>= 1) s[q] += __shfl_xor_sync(0xffffffffu, s[q], o);
    if (threadIdx.x == 0) {
        out[0] = s[0] * w0;
        out[1] = s[1] * w0 * mass;
        out[2] = s[2] * w0 * mass;
        out[3] = s[3] * w0 * mass;
        out[4] = 0.5 * mass * (w0 * s[4]);
    }
}

/* ======================================================================== */
static MixArgs mix_args(World &w, Species &s) {
    MixArgs a;
    a.ni = w.g.ni;
    a.nj = w.g.nj;
    a.nk = w.g.nk;
    a.qmdt = (float)(s.charge / s.mass * w.dt);
    for (int d = 0; d < 3; d++) {
        a.dtdh[d] = (float)(w.dt / w.g.dh[d]);
        a.dh[d] = (float)w.g.dh[d];
        a.sx[d] = (float)(w.g.x0[d] - w.sphere[d]);
    }
    a.r2 = w.has_sphere ? (float)w.sphere[3] : -1.f;
    return a;
}

/* the tile-segment push needs a whole box inside the grid */
static bool tiles_usable(const World &w, const Species &s) {
    return s.tiled && w.g.ni >= TBW && w.g.nj >= TBW && w.g.nk >= TBW;
}

template <int WALLS, bool DEP>
static void push_mixed_as(World &w, Species &s, int64_t n) {
    MixArgs a = mix_args(w, s);
    if (tiles_usable(w, s)) {
        const int64_t ntiles = (int64_t)tile_count(w.g.ni - 1) * tile_count(w.g.nj - 1) * tile_count(w.g.nk - 1);
        constexpr int BV = TBW * TBW * TBW;
        const int smem = BV * (int)sizeof(float4) + BV * (int)sizeof(unsigned int);
        /* the boxes take 44 KB of shared memory (set for the current device) */
        cudaFuncSetAttribute(k_push_tiles<WALLS, DEP>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (WALLS == M_ABSORB) /* the tile kernels OR their dead bits into the mask */
            cudaMemsetAsync(s.deadmask, 0, ((n + 31) / 32) * sizeof(uint32_t), w.stream);
        /* per-block sums of the pushed particles for the diagnostics row */
        const int64_t nsum = ntiles + 2 * (int64_t)w.sm_count;
        if (s.dsum_cap < nsum) {
            if (s.dsum) {
                cudaStreamSynchronize(w.stream);
                cudaFree(s.dsum);
            }
            s.dsum_cap = cudaMalloc(&s.dsum, 4 * nsum * sizeof(double)) == cudaSuccess ? nsum : 0;
            if (!s.dsum_cap) s.dsum = nullptr;
        }
        k_push_tiles<WALLS, DEP><<<(unsigned)ntiles, 256, smem, w.stream>>>(a, w.ef4, s.cell, s.off, s.vel, s.ms,
                                                                            s.seg, s.d_count, s.deadmask,
                                                                            s.tiledead, s.acc, w.d_err, s.dsum);
        k_push_tail<WALLS, DEP><<<2 * w.sm_count, 256, 0, w.stream>>>(a, w.ef4, s.cell, s.off, s.vel, s.ms,
                                                                       s.seg + ntiles, s.d_count, s.deadmask,
                                                                       s.tiledead, s.acc, w.d_err,
                                                                       s.dsum ? s.dsum + 4 * ntiles : nullptr);
        w.nlaunch += 2;
        s.dsum_n = s.dsum ? nsum : 0;
        s.dsum_valid = s.dsum != nullptr;
        return;
    }
    s.dsum_valid = false;
    k_push_mixed<WALLS, DEP><<<blocks_for(n, 256), 256, 0, w.stream>>>(a, w.ef4, s.cell, s.off, s.vel, s.ms,
                                                                      s.d_count, s.deadmask, s.tiledead, s.acc,
                                                                      w.d_err);
    w.nlaunch++;
}

void launch_push_mixed(World &w, Species &s, bool deposit) {
    int64_t n = s.host_bound;
    if (n <= 0) return;
    if (s.walls == 0) {
        if (deposit)
            push_mixed_as<M_REFLECT, true>(w, s, n);
        else
            push_mixed_as<M_REFLECT, false>(w, s, n);
    } else {
        if (deposit)
            push_mixed_as<M_ABSORB, true>(w, s, n);
        else
            push_mixed_as<M_ABSORB, false>(w, s, n);
    }
}

void launch_deposit_mixed(World &w, Species &s) {
    int64_t n = s.host_bound;
    if (n <= 0) return;
    MixArgs a = mix_args(w, s);
    if (tiles_usable(w, s)) {
        const int64_t ntiles = (int64_t)tile_count(w.g.ni - 1) * tile_count(w.g.nj - 1) * tile_count(w.g.nk - 1);
        k_deposit_tiles<<<(unsigned)ntiles, 256, 0, w.stream>>>(a, s.cell, s.off, s.ms, s.seg, s.d_count, s.acc);
        k_deposit_tail<<<2 * w.sm_count, 256, 0, w.stream>>>(a, s.cell, s.off, s.ms, s.seg + ntiles, s.d_count,
                                                             s.acc);
        w.nlaunch += 2;
        return;
    }
    k_deposit_mixed<<<blocks_for(n, 256), 256, 0, w.stream>>>(a, s.cell, s.off, s.ms, s.d_count, s.acc);
    w.nlaunch++;
}

void launch_to_mixed(World &w, Species &s, const double *P, int64_t stride, int64_t first, int64_t n) {
    s.dsum_valid = false;
    if (n <= 0) return;
    k_to_mixed<<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, P, stride, n, first, s.cell, s.off, s.vel,
                                                          s.ms);
    w.nlaunch++;
}

void launch_to_mixed_raw(cudaStream_t st, const Geo &g, const double *P, int64_t pstride, int64_t n, int64_t first,
                         int32_t *cell, float *off, float *vel, int64_t stride) {
    if (n <= 0) return;
    k_to_mixed<<<blocks_for(n, 256), 256, 0, st>>>(g, P, pstride, n, first, cell, off, vel, stride);
}

void launch_from_mixed_raw(cudaStream_t st, const Geo &g, const int32_t *cell, const float *off, const float *vel,
                           int64_t stride, int64_t first, int64_t n, double w0, double *P, int64_t pstride) {
    if (n <= 0) return;
    k_from_mixed_n<<<blocks_for(n, 256), 256, 0, st>>>(g, cell, off, vel, stride, first, n, w0, P, pstride);
}

void launch_from_mixed(World &w, Species &s, double *P, int64_t stride, int64_t n) {
    if (n <= 0) return;
    k_from_mixed<<<blocks_for(n, 256), 256, 0, w.stream>>>(w.g, s.cell, s.off, s.vel, s.ms, s.d_count, s.mpw0, P,
                                                           stride);
    w.nlaunch++;
}

void launch_sort_mixed(World &w, Species &s) {
    int64_t n = s.host_bound;
    if (n <= 0) return;
    const int ntx = tile_count(w.g.ni - 1), nty = tile_count(w.g.nj - 1), ntz = tile_count(w.g.nk - 1);
    const int64_t ntiles = (int64_t)ntx * nty * ntz;
    const int64_t ncells = ntiles * TILE_CELLS * TILE_CELLS * TILE_CELLS; /* slots of the tile-major order */
    int32_t *counts = s.sort_count;
    int32_t *bsum = counts + ncells + 1;
    int64_t nb = (ncells + SCAN_PER_BLOCK - 1) / SCAN_PER_BLOCK;
    cudaMemsetAsync(counts, 0, (ncells + 1) * sizeof(int32_t), w.stream);
    k_sort_hist<<<blocks_for(n, 256), 256, 0, w.stream>>>(s.cell, s.d_count, ntx, nty, counts);
    k_scan_reduce<<<(unsigned)nb, 1024, 0, w.stream>>>(counts, ncells, bsum);
    k_scan_bsum<<<1, 1024, 0, w.stream>>>(bsum, nb);
    k_scan_down<<<(unsigned)nb, 1024, 0, w.stream>>>(counts, ncells, bsum);
    k_tile_seg<<<blocks_for(ntiles + 1, 256), 256, 0, w.stream>>>(counts, ntiles, s.d_count, s.seg);
    k_sort_scatter<<<blocks_for(n, 256), 256, 0, w.stream>>>(s.cell, s.d_count, ntx, nty, counts, s.cell2);
    static bool carveout = false;
    if (!carveout) { /* no shared memory: the whole of it as L1 */
        cudaFuncSetAttribute(k_sort_gather_all, cudaFuncAttributePreferredSharedMemoryCarveout, 0);
        carveout = true;
    }
    k_sort_gather_all<<<blocks_for(n, GATHER_THREADS * GATHER_PER), GATHER_THREADS, 0, w.stream>>>(
        s.cell, s.off, s.vel, s.ms, s.d_count, s.cell2, s.off2, s.vel2, w.d_err);
    w.nlaunch += 7;
    s.tiled = true;
    int32_t *tc = s.cell;
    s.cell = s.cell2;
    s.cell2 = tc;
    float *to = s.off;
    s.off = s.off2;
    s.off2 = to;
    float *tv = s.vel;
    s.vel = s.vel2;
    s.vel2 = tv;
}

/* exclusive prefix sum of x[0..n) in place (bsum: int_scan_blocks(n) entries) */
int64_t int_scan_blocks(int64_t n) { return (n + SCAN_PER_BLOCK - 1) / SCAN_PER_BLOCK; }

void launch_int_excl_scan(cudaStream_t st, int32_t *x, int64_t n, int32_t *bsum) {
    const int64_t nb = int_scan_blocks(n);
    if (nb <= 0) return;
    k_scan_reduce<<<(unsigned)nb, 1024, 0, st>>>(x, n, bsum);
    k_scan_bsum<<<1, 1024, 0, st>>>(bsum, nb);
    k_scan_down<<<(unsigned)nb, 1024, 0, st>>>(x, n, bsum);
}

/* the diagnostics row from the push's per-block sums (sum v, sum |v|^2), in
 * block order, and the live count */
__global__ void k_dsum_final(const double *__restrict__ dsum, int64_t nb, const int64_t *__restrict__ d_count,
                             double mass, double w0, double *out) {
    __shared__ double ws[32][4];
    double t[4] = {0, 0, 0, 0};
    for (int64_t b = threadIdx.x; b < nb; b += blockDim.x)
        for (int q = 0; q < 4; q++) t[q] += dsum[4 * b + q];
    for (int q = 0; q < 4; q++)
        for (int o = 16; o > 0; o >>= 1) t[q] += __shfl_xor_sync(0xffffffffu, t[q], o);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 4; q++) ws[threadIdx.x >> 5][q] = t[q];
    __syncthreads();
    if (threadIdx.x == 0) {
        double s[4] = {0, 0, 0, 0};
        for (int w32 = 0; w32 < (int)(blockDim.x >> 5); w32++)
            for (int q = 0; q < 4; q++) s[q] += ws[w32][q];
        out[0] = (double)d_count[0] * w0;
        out[1] = s[0] * w0 * mass;
        out[2] = s[1] * w0 * mass;
        out[3] = s[2] * w0 * mass;
        out[4] = 0.5 * mass * (w0 * s[3]);
    }
}

/* first stage of the row's sums: block b adds its contiguous range of the
 * push's block sums (threads strided, then the warps in order), so that the
 * final kernel adds DSUM_PARTS partials instead of one per tile */
constexpr int DSUM_PARTS = 64;

__global__ void __launch_bounds__(256) k_dsum_part(const double *__restrict__ dsum, int64_t nb, double *part) {
    __shared__ double ws[8][4];
    const int64_t per = (nb + gridDim.x - 1) / gridDim.x;
    const int64_t b0 = (int64_t)blockIdx.x * per, b1 = b0 + per < nb ? b0 + per : nb;
    double t[4] = {0, 0, 0, 0};
    for (int64_t b = b0 + threadIdx.x; b < b1; b += blockDim.x)
        for (int q = 0; q < 4; q++) t[q] += dsum[4 * b + q];
    for (int q = 0; q < 4; q++)
        for (int o = 16; o > 0; o >>= 1) t[q] += __shfl_xor_sync(0xffffffffu, t[q], o);
    if ((threadIdx.x & 31) == 0)
        for (int q = 0; q < 4; q++) ws[threadIdx.x >> 5][q] = t[q];
    __syncthreads();
    if (threadIdx.x < 4) {
        double r = 0;
        for (int w8 = 0; w8 < (int)(blockDim.x >> 5); w8++) r += ws[w8][threadIdx.x];
        part[4 * (int64_t)blockIdx.x + threadIdx.x] = r;
    }
}

void launch_diag_mixed(World &w, Species &s, double *d_out5) {
    if (s.dsum_valid) { /* the sums the last push left (no particle has changed since) */
        if (s.dsum_n > 4 * DSUM_PARTS && w.partial_slots >= 4 * DSUM_PARTS) {
            k_dsum_part<<<DSUM_PARTS, 256, 0, w.stream>>>(s.dsum, s.dsum_n, w.d_partials);
            k_dsum_final<<<1, 1024, 0, w.stream>>>(w.d_partials, DSUM_PARTS, s.d_count, s.mass, s.mpw0, d_out5);
            w.nlaunch += 2;
        } else {
            k_dsum_final<<<1, 1024, 0, w.stream>>>(s.dsum, s.dsum_n, s.d_count, s.mass, s.mpw0, d_out5);
            w.nlaunch++;
        }
        return;
    }
    /* eight blocks of 256 per SM, within the partials buffer (5 per block) */
    int nb = 8 * w.sm_count;
    if (nb > w.partial_slots / 5) nb = w.partial_slots / 5;
    k_diag_mixed<<<nb, 256, 0, w.stream>>>(s.vel, s.ms, s.d_count, w.d_partials, nb);
    k_diag_mixed_final<<<1, 32, 0, w.stream>>>(w.d_partials, nb, s.mass, s.mpw0, d_out5);
    w.nlaunch += 2;
}

}  // namespace espic
