/*
 * k_pcg.cu -- matrix-free Newton / Jacobi-PCG solve of the Boltzmann-electron
 * Poisson problem of ch3/ver2 (PotentialSolver::solveNRPCG,
 * ch3/ver2/PotentialSolver.cpp:225-331), in one cooperative launch.
 *
 * The discrete problem is the one whose fixed point solveGS
 * (ch3/ver2/PotentialSolver.cpp:334-430) converges to.  Unknowns are the
 * interior nodes with object_id == 0.  With c = 1/dh^2 per axis,
 *   F_u = sum_{nb unknown or Dirichlet} c (phi_u - phi_nb)
 *         + (qe n0/eps0) exp((phi_u - phi0)/Te) - rho_u/eps0
 * (a Neumann boundary neighbour of an interior node always copies that node,
 * so it contributes nothing), and J = L + diag((qe n0/(eps0 Te)) e^...) is
 * symmetric positive definite.  The reference's own matrix has first-order,
 * non-symmetric Neumann rows on which CG breaks down.
 *
 * Newton residual F, the update of phi and the stopping test RMS(y) < nr_tol
 * (the reference's vec::norm, ch3/ver2/PotentialSolver.cpp:114-121) are
 * float64.  The inner PCG runs in T = double or float: with float it is the
 * inner solve of an iterative refinement whose outer residual is float64.
 * Dot products are reduced per block and summed by every block in block
 * order, so every block takes the same branch.  The inner PCG stops when
 * |r| <= pcg_tol |F|, or earlier once the RMS of the preconditioned residual
 * z = M r (an estimate of the error left in the Newton update y) is below
 * nr_tol / 2 (nr_tol / 10 in linear mode): the Newton test RMS(y) < nr_tol
 * cannot then depend on more inner accuracy, and the last Newton step stops
 * needing a full solve; when the first V-cycle's z is already that small,
 * z itself is the update.
 *
 * Preconditioner: an aggregation multigrid V-cycle.  Level l+1 groups the
 * level-l unknowns in 2x2x2 blocks of the structured index space; its
 * operator is the Galerkin product P^T A_l P with piecewise-constant P
 * (a 7-point stencil again, with per-node weights), built once per geometry
 * by a deterministic gather.  Smoothing is red-black Gauss-Seidel (red then
 * black before the coarse correction, black then red after), restriction is
 * P^T, prolongation P scaled by a constant.  The first level with at most
 * World::mg_dense_max nodes (default 1024) is the coarsest and is solved by
 * its dense inverse (computed once per geometry by k_gauss_jordan), every
 * level above it on the whole grid.  With mg_dense_max 0 (or a singular
 * coarse operator) the coarsest level gets symmetric sweeps instead and
 * levels with fewer than World::mg_block_nodes nodes (default 4096) run on
 * block 0 alone between two grid barriers.  Either way the preconditioner
 * is symmetric, as CG requires.  Without levels, it is Jacobi.
 */
#include <cooperative_groups.h>

#include "dfloat.h"
#include "espic_world.h"

namespace cg = cooperative_groups;

namespace espic {

#define PCG_EPS_0 8.85418782e-12
#define PCG_QE 1.602176565e-19

enum : uint16_t { SELF = 1u << 12, BLACK = 1u << 13 };

/* neighbour m: 0 -x, 1 +x, 2 -y, 3 +y, 4 -z, 5 +z.  bit m: unknown; bit 6+m:
 * Dirichlet; SELF: the node is an unknown. */
__global__ void k_pcg_codes(Geo g, const int32_t *__restrict__ obj, uint16_t *code) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
    uint16_t c = 0;
    bool interior = i > 0 && j > 0 && k > 0 && i < g.ni - 1 && j < g.nj - 1 && k < g.nk - 1;
    if (interior && obj[u] == 0) {
        c |= SELF;
        if ((i + j + k) & 1) c |= BLACK;
        int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
        int64_t nb[6] = {u - 1, u + 1, u - sy, u + sy, u - sz, u + sz};
        int ii[6] = {i - 1, i + 1, i, i, i, i}, jj[6] = {j, j, j - 1, j + 1, j, j},
            kk[6] = {k, k, k, k, k - 1, k + 1};
        for (int m = 0; m < 6; m++) {
            if (obj[nb[m]] > 0) {
                c |= (uint16_t)(1u << (6 + m));
            } else {
                bool in = ii[m] > 0 && jj[m] > 0 && kk[m] > 0 && ii[m] < g.ni - 1 && jj[m] < g.nj - 1 &&
                          kk[m] < g.nk - 1;
                if (in) c |= (uint16_t)(1u << m);
            }
        }
    }
    code[u] = c;
}

/* Grid-wide sums of NV values: block partials, one grid barrier, then every
 * block sums the partials with its first warp (lane l takes partials l,
 * l+32, ... in order; a fixed shuffle tree combines the lanes).  Every block
 * computes bit-identical totals, so all blocks take the same branches. */
template <int NV>
__device__ __forceinline__ void grid_sum_n(cg::grid_group &grid, double (&v)[NV], double *partials, int &round) {
    __shared__ double sh[NV][32];
    __shared__ double tot[NV];
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) sh[q][wid] = x;
    }
    __syncthreads();
    double *slot = partials + (size_t)(round & 1) * gridDim.x * NV;
    if (wid == 0) {
        /* the warps' sums by a fixed shuffle tree (blocks of 32 warps) */
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double s = lane < (int)(blockDim.x >> 5) ? sh[q][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) slot[(size_t)blockIdx.x * NV + q] = s;
        }
    }
    round++;
    grid.sync();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double s = 0;
#pragma unroll 4
            for (unsigned b = lane; b < gridDim.x; b += 32) s += __ldcg(slot + (size_t)b * NV + q);
            for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
            if (lane == 0) tot[q] = s;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = tot[q];
}


/* The same for per-thread values of the inner-solve type T: the warp stage
 * adds in T (for float, five float shuffle steps instead of five float64
 * ones in each of a block's 32 warps, which the narrow float64 pipe
 * serialised), then the warps' sums, the blocks' partials and the grid
 * total are float64 as above. */
template <int NV, typename T>
__device__ __forceinline__ void grid_sum_t(cg::grid_group &grid, const T (&v)[NV], double (&out)[NV],
                                           double *partials, int &round) {
    if (sizeof(T) == sizeof(double)) {
#pragma unroll
        for (int q = 0; q < NV; q++) out[q] = (double)v[q];
        grid_sum_n<NV>(grid, out, partials, round);
        return;
    }
    __shared__ double shw[NV][32];
    __shared__ double tot[NV];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; q++) {
        T x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if (lane == 0) shw[q][wid] = (double)x;
    }
    __syncthreads();
    double *slot = partials + (size_t)(round & 1) * gridDim.x * NV;
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double sum = lane < (int)(blockDim.x >> 5) ? shw[q][lane] : 0.0;
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            if (lane == 0) slot[(size_t)blockIdx.x * NV + q] = sum;
        }
    }
    round++;
    grid.sync();
    if (wid == 0) {
#pragma unroll
        for (int q = 0; q < NV; q++) {
            double sum = 0;
#pragma unroll 4
            for (unsigned b = lane; b < gridDim.x; b += 32) sum += __ldcg(slot + (size_t)b * NV + q);
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            if (lane == 0) tot[q] = sum;
        }
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; q++) out[q] = tot[q];
}

constexpr int MG_MAX = 12;
/* threads per block of the cooperative solve (one block per SM) */
constexpr int PCG_THREADS = 1024;
constexpr size_t PCG_SMEM_MAX = 160 * 1024; /* shared memory for block 0's coarse levels */

template <typename T>
struct MgLevel {
    int nx, ny, nz, pad;
    int64_t n;
    T *diag, *w, *b, *e; /* w: 6 weights per node, [m][n] */
};

template <typename T>
struct MgArgs {
    int nlev;        /* coarse levels (0: Jacobi preconditioner) */
    int grid_levels; /* coarse levels 1..grid_levels-1 run on the whole grid */
    int nu_coarse;   /* sweeps each way on the coarsest level */
    T scale;         /* coarse-correction scale */
    int smem_from;   /* block 0 keeps levels L[smem_from..] in shared memory (-1: none) */
    int dense_n;     /* nodes of the coarsest level when it is solved by its dense inverse */
    T *dense;        /* that inverse, row-major (null: smoothing sweeps on the coarsest level) */
    const int *dense_ok; /* 0 when the inversion met a vanishing pivot (a singular coarse operator,
                            e.g. without Dirichlet nodes): the coarsest level is smoothed instead */
    MgLevel<T> L[MG_MAX];
};

/* bytes of one level's arrays (diag, 6 weights, b, e) in shared memory */
template <typename T>
__host__ __device__ inline size_t level_smem_bytes(int64_t n) {
    return ((size_t)n * sizeof(T) + 15) / 16 * 16 * 9;
}

/* block 0's view of the levels it works alone: shared-memory copies of
 * L[smem_from..] (diag and weights copied once per launch) */
template <typename T>
__device__ void smem_levels_init(const MgArgs<T> &A, MgArgs<T> &S, unsigned char *base) {
    if (threadIdx.x == 0) {
        S = A;
        size_t off = 0;
        for (int i = A.smem_from; i < A.nlev; i++) {
            const int64_t n = A.L[i].n;
            const size_t a = ((size_t)n * sizeof(T) + 15) / 16 * 16;
            S.L[i].diag = (T *)(base + off);
            S.L[i].w = (T *)(base + off + a);
            S.L[i].b = (T *)(base + off + 7 * a);
            S.L[i].e = (T *)(base + off + 8 * a);
            off += 9 * a;
        }
    }
    __syncthreads();
    for (int i = A.smem_from; i < A.nlev; i++) {
        const int64_t n = A.L[i].n;
        for (int64_t t = threadIdx.x; t < n; t += blockDim.x) S.L[i].diag[t] = A.L[i].diag[t];
        for (int64_t t = threadIdx.x; t < 6 * n; t += blockDim.x) S.L[i].w[t] = A.L[i].w[t];
    }
    __syncthreads();
}

/* everything the level-0 (node grid) operations need */
template <typename T>
struct Coef3 {
    T c[3];
};

template <typename T>
struct Fine {
    Geo g;
    const uint16_t *code;
    T ct[3];
    int64_t off[6];
    T *dg, *r, *z; /* dg: the Boltzmann part of the Jacobian diagonal */
    const int32_t *list[2]; /* interior nodes of each colour (-1: padding) */
    const int32_t *pk[2];   /* their coordinates, i | j<<10 | k<<20 */
    int32_t nlist;          /* entries per list */
};

/* the interior nodes of colour c in a fixed order, with packed coordinates
 * (built once per geometry so that the sweeps need no division) */
__global__ void k_pcg_lists(Geo g, int c, int32_t *list, int32_t *pk) {
    int hx = (g.ni - 1) / 2;
    int64_t count = (int64_t)hx * (g.nj - 2) * (g.nk - 2);
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= count) return;
    int i2 = (int)(t % hx);
    int64_t rr = t / hx;
    int j = 1 + (int)(rr % (g.nj - 2));
    int k = 1 + (int)(rr / (g.nj - 2));
    int i = 1 + 2 * i2 + ((1 + j + k + c) & 1);
    if (i > g.ni - 2) {
        list[t] = -1;
        pk[t] = 0;
        return;
    }
    list[t] = (int32_t)(((int64_t)k * g.nj + j) * g.ni + i);
    pk[t] = i | (j << 10) | (k << 20);
}

__device__ __forceinline__ void span(bool whole, int64_t &t0, int64_t &ts) {
    if (whole) {
        t0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        ts = (int64_t)gridDim.x * blockDim.x;
    } else {
        t0 = threadIdx.x;
        ts = blockDim.x;
    }
}

/* Full Jacobian diagonal of an unknown: its Boltzmann part plus c per
 * unknown or Dirichlet neighbour. */
template <typename T>
__device__ __forceinline__ T full_diag(uint16_t cc, T dB, const T ct[3]) {
    T d = dB;
#pragma unroll
    for (int m = 0; m < 6; m++) d += (cc & ((1u << m) | (1u << (6 + m)))) ? ct[m >> 1] : (T)0;
    return d;
}

/* J x at an unknown in difference form, dB x_u + sum_unknown c (x_u - x_nb)
 * + sum_Dirichlet c x_u: no term is the difference of two large products,
 * so float keeps full relative accuracy on the smooth modes, where the
 * equivalent diag x_u - sum c x_nb loses most of its digits at fine spacing */
template <typename T>
__device__ __forceinline__ T jacobian_apply(uint16_t cc, T dB, const T ct[3], T xu, const T xn[6]) {
    T s = dB * xu;
#pragma unroll
    for (int m = 0; m < 6; m++)
        s += (cc & (1u << m)) ? ct[m >> 1] * (xu - xn[m]) : ((cc & (1u << (6 + m))) ? ct[m >> 1] * xu : (T)0);
    return s;
}

/* a node index clamped into the grid (loads of a boundary node's missing
 * neighbours, whose values are never used) */
__device__ __forceinline__ int64_t clamp_node(int64_t v, int64_t nn) { return v < 0 ? 0 : (v >= nn ? nn - 1 : v); }

/* red-black half sweep on the node grid: z = (r + sum c z_nb) / diag */
/* Red-black Gauss-Seidel pieces.  A Gauss-Seidel update never reads the
 * node's own old value, which allows three fusions: the first red half
 * sweep from a zero guess is pointwise (e = b / diag) and is done by whoever
 * produces b; the prolongation of the coarse correction is applied on the
 * fly to the red neighbours read by the following black half sweep (the red
 * nodes are overwritten next anyway); and the dot products r.z and z.z are
 * accumulated by the last two half sweeps, which produce the final z. */
/* node-grid half sweep of colour c over the unknowns; with C != null the
 * neighbours are read with the coarse correction added (post-smoothing);
 * adds r*z and z*z of the nodes it updated to rz and zz.  Each thread takes
 * two entries of the colour's enumeration per pass and issues every load of
 * both before any store (a padding entry reads the interior node (1,1,1) and
 * stores nothing), so twice as many loads are in flight as with one node per
 * pass.  Entry t is node i = 1 + 2 i2 + ((1+j+k+c)&1) of interior row
 * (j, k), with i2 = t mod hx; below 2^24 entries the coordinates come from
 * float-estimated divisions, above from the precomputed lists. */
template <typename T>
__device__ void fine_half(const Fine<T> &F, int c, const MgLevel<T> *C, T scale, T &rz_out, T &zz_out) {
    T rz = 0, zz = 0;
    int64_t t0, ts;
    span(true, t0, ts);
    const int32_t *list = F.list[c], *pk = F.pk[c];
    const Geo &g = F.g;
    const int64_t safe = ((int64_t)g.nj + 1) * g.ni + 1;
    const bool arith = F.nlist < (1 << 24);
    const uint32_t hx = (uint32_t)((g.ni - 1) / 2), rj = (uint32_t)(g.nj - 2);
    const float inv_hx = 1.f / (float)hx, inv_rj = 1.f / (float)rj;
    for (int64_t t = t0; t < F.nlist; t += 2 * ts) {
        const int64_t tq[2] = {t, t + ts};
        int64_t u[2];
        bool ok[2];
        int32_t pq[2];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (arith) {
                const bool in = tq[q] < F.nlist;
                const uint32_t tt = in ? (uint32_t)tq[q] : 0u;
                const uint32_t row = div_small(tt, hx, inv_hx);
                const uint32_t kk = div_small(row, rj, inv_rj);
                const int j = 1 + (int)(row - kk * rj), k = 1 + (int)kk;
                const int i = 1 + 2 * (int)(tt - row * hx) + ((1 + j + k + c) & 1);
                ok[q] = in && i <= g.ni - 2;
                u[q] = ok[q] ? ((int64_t)k * g.nj + j) * g.ni + i : safe;
                pq[q] = i | (j << 10) | (k << 20);
            } else {
                const int32_t uu = tq[q] < F.nlist ? list[tq[q]] : -1;
                ok[q] = uu >= 0;
                u[q] = ok[q] ? (int64_t)uu : safe;
                pq[q] = C && ok[q] ? pk[tq[q]] : 0;
            }
        }
        /* interior node: all six neighbours are in bounds, so their loads
         * are issued before the code word arrives; the code only selects */
        uint16_t cc[2];
        T ru[2], dBu[2], zn[2][6];
#pragma unroll
        for (int q = 0; q < 2; q++) {
            cc[q] = F.code[u[q]];
            ru[q] = F.r[u[q]];
            dBu[q] = F.dg[u[q]];
#pragma unroll
            for (int m = 0; m < 6; m++) zn[q][m] = F.z[u[q] + F.off[m]];
        }
        if (C) {
            /* the coarse correction at the six neighbours: for each axis one
             * neighbour shares the node's aggregate, the other is the next
             * aggregate on the side of the node's parity */
            const MgLevel<T> &Cc = *C;
            T ea[2], ex[2], ey[2], ez[2];
            int par[2];
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const int32_t p = ok[q] ? pq[q] : (1 | (1 << 10) | (1 << 20));
                const int i = p & 1023, j = (p >> 10) & 1023, k = p >> 20;
                const int32_t sy = Cc.nx, sz = Cc.nx * Cc.ny;
                const int32_t A = ((k >> 1) * Cc.ny + (j >> 1)) * Cc.nx + (i >> 1);
                par[q] = (i & 1) | ((j & 1) << 1) | ((k & 1) << 2);
                ea[q] = Cc.e[A];
                ex[q] = Cc.e[(i & 1) ? A + 1 : A - 1];
                ey[q] = Cc.e[(j & 1) ? A + sy : A - sy];
                ez[q] = Cc.e[(k & 1) ? A + sz : A - sz];
            }
#pragma unroll
            for (int q = 0; q < 2; q++) {
                const bool oi = par[q] & 1, oj = par[q] & 2, ok_ = par[q] & 4;
                zn[q][0] += scale * (oi ? ea[q] : ex[q]);
                zn[q][1] += scale * (oi ? ex[q] : ea[q]);
                zn[q][2] += scale * (oj ? ea[q] : ey[q]);
                zn[q][3] += scale * (oj ? ey[q] : ea[q]);
                zn[q][4] += scale * (ok_ ? ea[q] : ez[q]);
                zn[q][5] += scale * (ok_ ? ez[q] : ea[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 2; q++) {
            if (!ok[q] || !(cc[q] & SELF)) continue;
            T s = ru[q];
#pragma unroll
            for (int m = 0; m < 6; m++) s += (cc[q] & (1u << m)) ? F.ct[m >> 1] * zn[q][m] : (T)0;
            const T zu = s / full_diag(cc[q], dBu[q], F.ct);
            F.z[u[q]] = zu;
            rz += ru[q] * zu;
            zz += zu * zu;
        }
    }
    rz_out += rz;
    zz_out += zz;
}

/* one half sweep of colour c on a coarse level; with C != null the
 * neighbours are read with C's correction added.  Coordinates come from the
 * sweep index by float-estimated divisions (levels below 2^24 nodes), the
 * neighbours' aggregates from the coordinates. */
template <typename T>
__device__ void coarse_half(const MgLevel<T> &L, int c, bool whole, const MgLevel<T> *C, T scale) {
    const int hx = (L.nx + 1) / 2;
    const int64_t count = (int64_t)hx * L.ny * L.nz;
    const int64_t offs[6] = {-1, 1, -(int64_t)L.nx, L.nx, -(int64_t)L.nx * L.ny, (int64_t)L.nx * L.ny};
    const bool fast = count < (1 << 24);
    const float inv_hx = 1.f / (float)hx, inv_ny = 1.f / (float)L.ny;
    int64_t t0, ts;
    span(whole, t0, ts);
    for (int64_t t = t0; t < count; t += ts) {
        const uint32_t tt = (uint32_t)t;
        uint32_t rr, kk;
        if (fast) {
            rr = div_small(tt, (uint32_t)hx, inv_hx);
            kk = div_small(rr, (uint32_t)L.ny, inv_ny);
        } else {
            rr = tt / (uint32_t)hx;
            kk = rr / (uint32_t)L.ny;
        }
        const int i2 = (int)(tt - rr * (uint32_t)hx);
        const int j = (int)(rr - kk * (uint32_t)L.ny);
        const int k = (int)kk;
        const int i = 2 * i2 + ((j + k + c) & 1);
        if (i >= L.nx) continue;
        const int64_t I = ((int64_t)k * L.ny + j) * L.nx + i;
        /* all loads first (a missing neighbour reads a clamped node; its zero
         * weight deselects it), then the arithmetic */
        T d = L.diag[I];
        T s = L.b[I];
        T wm[6], en[6];
        const int ci[6] = {i > 0 ? i - 1 : 0, i + 1 < L.nx ? i + 1 : i, i, i, i, i};
        const int cj[6] = {j, j, j > 0 ? j - 1 : 0, j + 1 < L.ny ? j + 1 : j, j, j};
        const int ck[6] = {k, k, k, k, k > 0 ? k - 1 : 0, k + 1 < L.nz ? k + 1 : k};
#pragma unroll
        for (int m = 0; m < 6; m++) {
            int64_t nb = I + offs[m];
            nb = nb < 0 ? 0 : (nb >= L.n ? L.n - 1 : nb);
            wm[m] = L.w[m * L.n + I];
            en[m] = L.e[nb];
            if (C) en[m] += scale * C->e[((ck[m] >> 1) * C->ny + (cj[m] >> 1)) * C->nx + (ci[m] >> 1)];
        }
        if (d == (T)0) continue;
#pragma unroll
        for (int m = 0; m < 6; m++) s += (wm[m] != (T)0) ? wm[m] * en[m] : (T)0;
        L.e[I] = s / d;
    }
}

/* The red children of a coarse node (its 2x2x2 block), in the order in which
 * their residuals are summed: offsets dx | dy<<1 | dz<<2 with dx+dy+dz even
 * (black residuals are zero after the black half sweep). */
__device__ __forceinline__ int red_child(int q) { return q == 0 ? 0 : (q == 1 ? 3 : (q == 2 ? 5 : 6)); }

/* Coordinates of coarse node I (float-estimated divisions below 2^24 nodes). */
template <typename T>
__device__ __forceinline__ void coarse_coords(const MgLevel<T> &C, int64_t I, bool fast, float inv_nx, float inv_ny,
                                              int &ci, int &cj, int &ck) {
    const uint32_t I32 = (uint32_t)I;
    const uint32_t cr = fast ? div_small(I32, (uint32_t)C.nx, inv_nx) : I32 / (uint32_t)C.nx;
    const uint32_t ckk = fast ? div_small(cr, (uint32_t)C.ny, inv_ny) : cr / (uint32_t)C.ny;
    ci = (int)(I32 - cr * (uint32_t)C.nx);
    cj = (int)(cr - ckk * (uint32_t)C.ny);
    ck = (int)ckk;
}

/* The sum of four lanes' residuals (lanes 4g..4g+3, in lane order) into
 * b of the coarse node, and the fused first red half sweep (e = b / diag).
 * Every lane of the warp calls it. */
template <typename T>
__device__ __forceinline__ void restrict_store(const MgLevel<T> &C, bool valid, int64_t I, int ci, int cj, int ck,
                                               T res) {
    const T r1 = __shfl_down_sync(0xffffffffu, res, 1);
    const T r2 = __shfl_down_sync(0xffffffffu, res, 2);
    const T r3 = __shfl_down_sync(0xffffffffu, res, 3);
    if (!valid || (threadIdx.x & 3)) return;
    T sum = 0;
    sum += res;
    sum += r1;
    sum += r2;
    sum += r3;
    C.b[I] = sum;
    if (((ci + cj + ck) & 1) == 0) {
        const T d = C.diag[I];
        if (d != (T)0) C.e[I] = sum / d;
    }
}

/* b of level 1 = sum of the node-grid children's residuals (r - J z).  When
 * the level has fewer nodes than the grid has threads (latency-bound),
 * four consecutive threads take the four red children of a coarse node,
 * each issuing all its loads at once (neighbour indices clamped into the
 * grid; a child that is not an unknown contributes zero); otherwise
 * (bandwidth-bound) a thread takes a coarse node and its four children, so
 * that a warp's loads of one child cover consecutive nodes of a row. */
template <typename T>
__device__ void restrict_fine(const Fine<T> &F, const MgLevel<T> &C) {
    const Geo &g = F.g;
    const int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    const int64_t safe = ((int64_t)g.nj + 1) * g.ni + 1;
    int64_t t0, ts;
    span(true, t0, ts);
    const bool fast = C.n < (1 << 24);
    const float inv_nx = 1.f / (float)C.nx, inv_ny = 1.f / (float)C.ny;
    if (C.n > ts) {
        for (int64_t I = t0; I < C.n; I += ts) {
            int ci, cj, ck;
            coarse_coords(C, I, fast, inv_nx, inv_ny, ci, cj, ck);
            T sum = 0;
            int64_t uu[4];
            uint16_t cc[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int d = red_child(q);
                const int i = 2 * ci + (d & 1), j = 2 * cj + ((d >> 1) & 1), k = 2 * ck + (d >> 2);
                const bool in = i < g.ni && j < g.nj && k < g.nk;
                uu[q] = in ? ((int64_t)k * g.nj + j) * g.ni + i : 0;
                cc[q] = in ? F.code[uu[q]] : (uint16_t)0;
            }
#pragma unroll
            for (int q = 0; q < 4; q++) {
                if (!(cc[q] & SELF)) continue;
                const int64_t u = uu[q];
                T zn[6];
#pragma unroll
                for (int m = 0; m < 6; m++) zn[m] = F.z[u + F.off[m]];
                sum += F.r[u] - jacobian_apply(cc[q], F.dg[u], F.ct, F.z[u], zn);
            }
            C.b[I] = sum;
            if (((ci + cj + ck) & 1) == 0) {
                const T d = C.diag[I];
                if (d != (T)0) C.e[I] = sum / d;
            }
        }
        return;
    }
    const int64_t total = 4 * C.n, padded = (total + 31) & ~(int64_t)31;
    for (int64_t t = t0; t < padded; t += ts) {
        const bool valid = t < total;
        const int64_t I = valid ? (t >> 2) : 0;
        int ci, cj, ck;
        coarse_coords(C, I, fast, inv_nx, inv_ny, ci, cj, ck);
        const int d = red_child((int)(t & 3));
        const int i = 2 * ci + (d & 1), j = 2 * cj + ((d >> 1) & 1), k = 2 * ck + (d >> 2);
        const bool in = valid && i < g.ni && j < g.nj && k < g.nk;
        const int64_t u = in ? ((int64_t)k * g.nj + j) * g.ni + i : safe;
        const uint16_t cc = F.code[u];
        const T ru = F.r[u], dBu = F.dg[u], zu = F.z[u];
        T zn[6];
#pragma unroll
        for (int m = 0; m < 6; m++) {
            int64_t nb = u + F.off[m];
            nb = nb < 0 ? 0 : (nb >= nn ? nn - 1 : nb);
            zn[m] = F.z[nb];
        }
        const T res = (in && (cc & SELF)) ? ru - jacobian_apply(cc, dBu, F.ct, zu, zn) : (T)0;
        restrict_store(C, valid, I, ci, cj, ck, res);
    }
}

/* b of level l+1 from level l, laid out like restrict_fine */
template <typename T>
__device__ void restrict_coarse(const MgLevel<T> &L, const MgLevel<T> &C, bool whole) {
    const int64_t offs[6] = {-1, 1, -(int64_t)L.nx, L.nx, -(int64_t)L.nx * L.ny, (int64_t)L.nx * L.ny};
    int64_t t0, ts;
    span(whole, t0, ts);
    const bool fast = C.n < (1 << 24);
    const float inv_nx = 1.f / (float)C.nx, inv_ny = 1.f / (float)C.ny;
    if (C.n > ts) {
        for (int64_t I = t0; I < C.n; I += ts) {
            int ci, cj, ck;
            coarse_coords(C, I, fast, inv_nx, inv_ny, ci, cj, ck);
            T sum = 0;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const int d = red_child(q);
                const int i = 2 * ci + (d & 1), j = 2 * cj + ((d >> 1) & 1), k = 2 * ck + (d >> 2);
                const bool in = i < L.nx && j < L.ny && k < L.nz;
                const int64_t u = in ? ((int64_t)k * L.ny + j) * L.nx + i : 0;
                const T dd = L.diag[u], bu = L.b[u], eu = L.e[u];
                T wm[6], en[6];
#pragma unroll
                for (int m = 0; m < 6; m++) {
                    int64_t nb = u + offs[m];
                    nb = nb < 0 ? 0 : (nb >= L.n ? L.n - 1 : nb);
                    wm[m] = L.w[m * L.n + u];
                    en[m] = L.e[nb];
                }
                if (!in || dd == (T)0) continue;
                T res = bu - dd * eu;
#pragma unroll
                for (int m = 0; m < 6; m++) res += (wm[m] != (T)0) ? wm[m] * en[m] : (T)0;
                sum += res;
            }
            C.b[I] = sum;
            if (((ci + cj + ck) & 1) == 0) {
                const T d = C.diag[I];
                if (d != (T)0) C.e[I] = sum / d;
            }
        }
        return;
    }
    const int64_t total = 4 * C.n, padded = (total + 31) & ~(int64_t)31;
    for (int64_t t = t0; t < padded; t += ts) {
        const bool valid = t < total;
        const int64_t I = valid ? (t >> 2) : 0;
        int ci, cj, ck;
        coarse_coords(C, I, fast, inv_nx, inv_ny, ci, cj, ck);
        const int d = red_child((int)(t & 3));
        const int i = 2 * ci + (d & 1), j = 2 * cj + ((d >> 1) & 1), k = 2 * ck + (d >> 2);
        const bool in = valid && i < L.nx && j < L.ny && k < L.nz;
        const int64_t u = in ? ((int64_t)k * L.ny + j) * L.nx + i : 0;
        const T dd = L.diag[u], bu = L.b[u], eu = L.e[u];
        T wm[6], en[6];
#pragma unroll
        for (int m = 0; m < 6; m++) {
            int64_t nb = u + offs[m];
            nb = nb < 0 ? 0 : (nb >= L.n ? L.n - 1 : nb);
            wm[m] = L.w[m * L.n + u];
            en[m] = L.e[nb];
        }
        T res = 0;
        if (in && dd != (T)0) {
            res = bu - dd * eu;
#pragma unroll
            for (int m = 0; m < 6; m++) res += (wm[m] != (T)0) ? wm[m] * en[m] : (T)0;
        }
        restrict_store(C, valid, I, ci, cj, ck, res);
    }
}

/* e = A^-1 b on the coarsest level by its dense inverse, on the whole grid:
 * block b takes a contiguous range of rows, eight at a time, four warps per
 * row, each warp a quarter of the columns (lanes in a fixed order, a fixed
 * shuffle tree); the four quarter sums are added in order.  Every thread of
 * every block calls it (blocks of 128 threads or a multiple). */
template <typename T>
__device__ void dense_apply(const MgLevel<T> &L, const T *__restrict__ Ainv, int n) {
    __shared__ T part[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int WPR = 4; /* warps per row */
    const int RPP = (int)(blockDim.x >> 5) / WPR; /* rows per pass */
    const int64_t rpb = ((int64_t)n + gridDim.x - 1) / gridDim.x;
    const int64_t r0 = (int64_t)blockIdx.x * rpb;
    const int64_t r1 = r0 + rpb < n ? r0 + rpb : n;
    for (int64_t rb = r0; rb < r1; rb += RPP) {
        const int64_t r = rb + wid / WPR;
        const int q = wid % WPR;
        T acc = 0;
        if (r < r1) {
            const int64_t c0 = (int64_t)q * n / WPR, c1 = (int64_t)(q + 1) * n / WPR;
            const T *row = Ainv + r * n;
#pragma unroll 8
            for (int64_t j = c0 + lane; j < c1; j += 32) acc += row[j] * L.b[j];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) part[wid] = acc;
        __syncthreads();
        if (threadIdx.x < RPP && rb + threadIdx.x < r1) {
            T sum = 0;
#pragma unroll
            for (int k = 0; k < WPR; k++) sum += part[threadIdx.x * WPR + k];
            L.e[rb + threadIdx.x] = sum;
        }
        __syncthreads();
    }
}

/* The V-cycle z = M r after its first red half sweep on the node grid
 * (done by the caller, fused with the CG update of r).  Every block executes
 * the same grid barriers; returns the grid-wide r.z of the final z and puts
 * z.z in zz (the last barrier is the one of that reduction). */
template <typename T>
__device__ double vcycle_rest(cg::grid_group &grid, const Fine<T> &F, const MgArgs<T> &A, double *partials,
                              int &round, double &zz, const MgArgs<T> *SB) {
    const int NL = A.nlev;
    if (NL == 0) { /* Jacobi: the caller computed z on every node */
        T rz = 0, z2 = 0;
        int64_t nn = (int64_t)F.g.ni * F.g.nj * F.g.nk;
        int64_t t0, ts;
        span(true, t0, ts);
        for (int64_t u = t0; u < nn; u += ts)
            if (F.code[u] & SELF) {
                T zu = F.z[u];
                rz += F.r[u] * zu;
                z2 += zu * zu;
            }
        const T vt[2] = {rz, z2};
        double v[2];
        grid_sum_t<2, T>(grid, vt, v, partials, round);
        zz = v[1];
        return v[0];
    }
    const int GL = A.grid_levels;
    const T sc = A.scale;
    T rz = 0, z2 = 0, rz_unused = 0, z2_unused = 0;
    fine_half(F, 1, (const MgLevel<T> *)nullptr, sc, rz_unused, z2_unused);
    grid.sync();
    restrict_fine(F, A.L[0]);
    grid.sync();
    int l = 1; /* level l lives in A.L[l-1] and its red half was fused */
    for (; l < GL && l < NL; l++) {
        coarse_half(A.L[l - 1], 1, true, (const MgLevel<T> *)nullptr, sc);
        grid.sync();
        restrict_coarse(A.L[l - 1], A.L[l], true);
        grid.sync();
    }
    const int lblock = l;
    const bool coarsest_whole = NL < GL;
    const int nuc = A.nu_coarse;
    if (!coarsest_whole) {
        if (blockIdx.x == 0) {
            /* with shared-memory levels, stage b and e of the first one */
            const bool staged = SB && SB->smem_from == lblock - 1;
            const MgArgs<T> &B = staged ? *SB : A;
            if (staged) {
                const MgLevel<T> &G0 = A.L[lblock - 1], &S0 = SB->L[lblock - 1];
                for (int64_t t = threadIdx.x; t < G0.n; t += blockDim.x) {
                    S0.b[t] = G0.b[t];
                    S0.e[t] = G0.e[t];
                }
                __syncthreads();
            }
            for (int b = lblock; b < NL; b++) {
                coarse_half(B.L[b - 1], 1, false, (const MgLevel<T> *)nullptr, sc);
                __syncthreads();
                restrict_coarse(B.L[b - 1], B.L[b], false);
                __syncthreads();
            }
            const MgLevel<T> &Lc = B.L[NL - 1];
            for (int s = 0; s < nuc; s++) {
                if (s) {
                    coarse_half(Lc, 0, false, (const MgLevel<T> *)nullptr, sc);
                    __syncthreads();
                }
                coarse_half(Lc, 1, false, (const MgLevel<T> *)nullptr, sc);
                __syncthreads();
            }
            for (int s = 0; s < nuc; s++) {
                coarse_half(Lc, 1, false, (const MgLevel<T> *)nullptr, sc);
                __syncthreads();
                coarse_half(Lc, 0, false, (const MgLevel<T> *)nullptr, sc);
                __syncthreads();
            }
            for (int b = NL - 1; b >= lblock; b--) {
                coarse_half(B.L[b - 1], 1, false, &B.L[b], sc);
                __syncthreads();
                coarse_half(B.L[b - 1], 0, false, (const MgLevel<T> *)nullptr, sc);
                __syncthreads();
            }
            if (staged) {
                const MgLevel<T> &G0 = A.L[lblock - 1], &S0 = SB->L[lblock - 1];
                for (int64_t t = threadIdx.x; t < G0.n; t += blockDim.x) G0.e[t] = S0.e[t];
            }
        }
        grid.sync();
    } else if (A.dense && *A.dense_ok) {
        dense_apply(A.L[NL - 1], A.dense, A.dense_n);
        grid.sync();
    } else {
        const MgLevel<T> &Lc = A.L[NL - 1];
        for (int s = 0; s < nuc; s++) {
            if (s) {
                coarse_half(Lc, 0, true, (const MgLevel<T> *)nullptr, sc);
                grid.sync();
            }
            coarse_half(Lc, 1, true, (const MgLevel<T> *)nullptr, sc);
            grid.sync();
        }
        for (int s = 0; s < nuc; s++) {
            coarse_half(Lc, 1, true, (const MgLevel<T> *)nullptr, sc);
            grid.sync();
            coarse_half(Lc, 0, true, (const MgLevel<T> *)nullptr, sc);
            grid.sync();
        }
    }
    const int top = coarsest_whole ? NL - 1 : lblock - 1;
    for (int b = top; b >= 1; b--) {
        coarse_half(A.L[b - 1], 1, true, &A.L[b], sc);
        grid.sync();
        coarse_half(A.L[b - 1], 0, true, (const MgLevel<T> *)nullptr, sc);
        grid.sync();
    }
    fine_half(F, 1, &A.L[0], sc, rz, z2);
    grid.sync();
    fine_half(F, 0, (const MgLevel<T> *)nullptr, sc, rz, z2);
    const T vt[2] = {rz, z2};
    double v[2];
    grid_sum_t<2, T>(grid, vt, v, partials, round);
    zz = v[1];
    return v[0];
}



/* The pairs of phi and rho / eps0 at every node, once per solve, with the
 * predictor folded in.  phi_prev holds two rows, the potentials of the last
 * two solves before this one (p1 = phi_prev, p2 = phi_prev + nn); phi is
 * the last solve's.  predict 1: p1 = phi; 2: also start each unknown from
 * 2 phi - p1 (linear extrapolation in time), and p2 = p1; 3: start from
 * 3 phi - 3 p1 + p2 (quadratic), and p2 = p1.  In double-float. */
__device__ __noinline__ void df_prepass(const double *__restrict__ phi, const double *__restrict__ rho, float2 *phf,
                                        float2 *rhf, const uint16_t *__restrict__ code, double *phi_prev,
                                        int predict, dfl d_inv_eps0, int64_t nn, int64_t gtid, int64_t gsize) {
    /* four nodes a pass, every load before any store (the pass is bound by
     * the loads in flight) */
    for (int64_t u0 = gtid; u0 < nn; u0 += 4 * gsize) {
        double cur[4], prev[4], prev2[4], rh[4];
        uint16_t c[4];
        bool on[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int64_t u = u0 + h * gsize;
            on[h] = u < nn;
            const int64_t v = on[h] ? u : 0;
            cur[h] = phi[v];
            rh[h] = rho[v];
            c[h] = predict >= 2 ? code[v] : (uint16_t)0;
            prev[h] = predict >= 2 ? phi_prev[v] : 0.0;
            prev2[h] = predict == 3 ? phi_prev[nn + v] : 0.0;
        }
#pragma unroll
        for (int h = 0; h < 4; h++) {
            if (!on[h]) continue;
            const int64_t u = u0 + h * gsize;
            dfl x = df_split(cur[h]);
            if (predict) {
                if (predict >= 2 && (c[h] & SELF)) {
                    const dfl p1 = df_split(prev[h]);
                    if (predict == 2) {
                        x = df_add({2.f * x.h, 2.f * x.l}, df_neg(p1));
                    } else {
                        const dfl d = df_add(x, df_neg(p1));
                        x = df_add({3.f * d.h, 3.f * d.l}, df_split(prev2[h]));
                    }
                }
                if (predict >= 2) phi_prev[nn + u] = prev[h];
                phi_prev[u] = cur[h];
            }
            phf[u] = df_pack(x);
            rhf[u] = df_pack(df_mul(df_split(rh[h]), d_inv_eps0));
        }
    }
}

/* The Newton update phi -= y on the pairs of the unknowns; returns the
 * thread's sum of y^2 */
template <typename T>
__device__ __noinline__ float df_update(const uint16_t *__restrict__ code, const T *__restrict__ yv, float2 *phf,
                                        int64_t nn, int64_t gtid, int64_t gsize) {
    float yys = 0.f;
    /* four nodes a pass, every load before any store */
    for (int64_t u0 = gtid; u0 < nn; u0 += 4 * gsize) {
        uint16_t c[4];
        float yu[4];
        float2 x[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int64_t u = u0 + h * gsize;
            const int64_t v = u < nn ? u : 0;
            c[h] = u < nn ? code[v] : (uint16_t)0;
            yu[h] = (float)yv[v];
            x[h] = phf[v];
        }
#pragma unroll
        for (int h = 0; h < 4; h++) {
            if (!(c[h] & SELF)) continue;
            phf[u0 + h * gsize] = df_pack(df_add(df_unpack(x[h]), {-yu[h], 0.f}));
            yys = __fmaf_rn(yu[h], yu[h], yys);
        }
    }
    return yys;
}

/* phi of the unknowns from their pairs (hi + lo rounded once), four nodes
 * a pass with every load before any store */
__device__ __noinline__ void df_rebuild(const uint16_t *__restrict__ code, const float2 *__restrict__ phf,
                                        double *phi, int64_t nn, int64_t gtid, int64_t gsize) {
    for (int64_t u0 = gtid; u0 < nn; u0 += 4 * gsize) {
        uint16_t c[4];
        float2 x[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int64_t u = u0 + h * gsize;
            c[h] = u < nn ? code[u] : (uint16_t)0;
            x[h] = phf[u < nn ? u : 0];
        }
#pragma unroll
        for (int h = 0; h < 4; h++)
            if (c[h] & SELF) phi[u0 + h * gsize] = (double)x[h].x + (double)x[h].y;
    }
}

/* Neumann boundary nodes take the value at the end of their chain (the
 * chains end at unknowns or Dirichlet nodes, which this pass does not
 * write), four nodes a pass */
__device__ __noinline__ void neumann_copies(const int32_t *__restrict__ target, double *phi, int64_t nn,
                                            int64_t gtid, int64_t gsize) {
    for (int64_t u0 = gtid; u0 < nn; u0 += 4 * gsize) {
        int32_t t[4];
#pragma unroll
        for (int h = 0; h < 4; h++) {
            const int64_t u = u0 + h * gsize;
            t[h] = u < nn ? target[u] : -1;
        }
#pragma unroll
        for (int h = 0; h < 4; h++)
            if (t[h] >= 0) phi[u0 + h * gsize] = phi[t[h]];
    }
}

/* The Newton residual pass of the float-inner nonlinear solve in
 * double-float arithmetic (per axis c (2 x_u - x_w - x_e), a missing link
 * reading x_u; the Boltzmann factor as expf of the leading part times a
 * first-order factor for the rest; rho / eps0 from its pair), with the
 * Jacobian's Boltzmann diagonal and the first red smoothing half sweep.
 * Returns the thread's sum of r^2.  Not inlined: the call spills the
 * solver's live state once, and the loop gets the registers (inlined, the
 * loop ran 4x slower).  An unknown is an interior node, so its neighbours
 * need no clamp (s1, s2: the y and z strides). */
template <typename T>
__device__ __noinline__ float df_residual(const uint16_t *__restrict__ code, const float2 *__restrict__ phf,
                                          const float2 *__restrict__ rhf, T *z, T *dg, T *r, T *y, int64_t nn,
                                          int64_t gtid, int64_t gsize, int32_t s1, int32_t s2, const T ct[3],
                                          const float cl[3], dfl d_phi0, dfl d_inv_te0, dfl d_A0, float A0_te0,
                                          bool jacobi) {
    float ffs = 0.f;
    /* two nodes a pass, every load before the arithmetic; a node that is
     * not an unknown reads the interior node safe_u and stores nothing */
    const int64_t safe_u = (int64_t)s2 + s1 + 1;
    for (int64_t u0 = gtid; u0 < nn; u0 += 2 * gsize) {
        uint16_t cq[2];
        int64_t uq[2];
        float2 xq[2], pq[2][6], bq[2];
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int64_t u = u0 + h * gsize;
            cq[h] = u < nn ? code[u] : (uint16_t)0;
            uq[h] = (cq[h] & SELF) ? u : safe_u;
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const float2 *pu = phf + uq[h];
            xq[h] = pu[0];
            pq[h][0] = pu[-1];
            pq[h][1] = pu[1];
            pq[h][2] = pu[-s1];
            pq[h][3] = pu[s1];
            pq[h][4] = pu[-s2];
            pq[h][5] = pu[s2];
            bq[h] = rhf[uq[h]];
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const uint16_t c = cq[h];
            if (!(c & SELF)) continue;
            const int64_t u = uq[h];
            const float2 xu = xq[h];
            const dfl x = df_unpack(xu);
            dfl L = {0.f, 0.f};
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const unsigned mw = (1u << (2 * a)) | (1u << (6 + 2 * a));
                const unsigned me = (1u << (2 * a + 1)) | (1u << (7 + 2 * a));
                const dfl pw = df_unpack((c & mw) ? pq[h][2 * a] : xu);
                const dfl pe = df_unpack((c & me) ? pq[h][2 * a + 1] : xu);
                const dfl d = df_add(df_add({2.f * x.h, 2.f * x.l}, df_neg(pw)), df_neg(pe));
                L = df_add(L, df_mul(d, {(float)ct[a], cl[a]}));
            }
            const dfl xa = df_mul(df_add(x, df_neg(d_phi0)), d_inv_te0);
            const float ef = expf(xa.h);
            const dfl e = df_fast2(ef, ef * xa.l);
            const dfl Fd = df_add(df_add(L, df_mul(d_A0, e)), df_neg(df_unpack(bq[h])));
            const float rv = Fd.h + Fd.l;
            const float dBt = A0_te0 * ef;
            if (jacobi || !(c & BLACK)) z[u] = (T)(rv / full_diag(c, (T)dBt, ct));
            dg[u] = (T)dBt;
            r[u] = (T)rv;
            y[u] = 0;
            ffs = __fmaf_rn(rv, rv, ffs);
        }
    }
    return ffs;
}

template <typename T>
__global__ void __launch_bounds__(PCG_THREADS, 1) k_newton_pcg(Geo g, double *phi, const double *__restrict__ rho,
                                                        const uint16_t *__restrict__ code,
                                                        const int32_t *__restrict__ target, double phi0,
                                                        double te0, double n0, int nr_max, double nr_tol,
                                                        int pcg_max, double pcg_tol, T *y, T *r, T *z, T *p0,
                                                        T *p1, T *q, T *dg, MgArgs<T> mg, const int32_t *lists,
                                                        double *partials, SolveStatus *st, int *err,
                                                        double *lin_y, const double *__restrict__ lin_b,
                                                        int gs_max, double gs_tol, float2 *dfbuf, double *phi_prev,
                                                        int predict, Coef3<T> ctp) {
    cg::grid_group grid = cg::this_grid();
    extern __shared__ __align__(16) unsigned char pcg_smem[];
    __shared__ T bc_alpha, bc_beta;
    __shared__ int bc_stop;
    __shared__ MgArgs<T> smem_args;
    const MgArgs<T> *SB = nullptr;
    if (mg.smem_from >= 0 && mg.nlev > 0 && blockIdx.x == 0) {
        smem_levels_init(mg, smem_args, pcg_smem);
        SB = &smem_args;
    }
    const int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    const int64_t off[6] = {-1, 1, -sy, sy, -sz, sz};
    const int64_t safe = sz + sy + 1; /* the interior node (1,1,1) */
    const double cd[3] = {1.0 / (g.dh[0] * g.dh[0]), 1.0 / (g.dh[1] * g.dh[1]), 1.0 / (g.dh[2] * g.dh[2])};
    /* (T)cd from the host: derived here from cd, the compiler re-derived it
     * inside the node loops (a float64-to-float conversion each time, on the
     * narrow float64 pipe) instead of holding it */
    const bool tf = sizeof(T) == sizeof(float);
    const T ct[3] = {tf ? ctp.c[0] : (T)cd[0], tf ? ctp.c[1] : (T)cd[1], tf ? ctp.c[2] : (T)cd[2]};
    const double A0 = PCG_QE * n0 / PCG_EPS_0;
    const double inv_te0 = 1.0 / te0, A0_te0 = A0 / te0, inv_eps0 = 1.0 / PCG_EPS_0;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
    const bool jacobi = mg.nlev == 0;
    Fine<T> F;
    F.g = g;
    F.code = code;
    for (int m = 0; m < 3; m++) F.ct[m] = ct[m];
    for (int m = 0; m < 6; m++) F.off[m] = off[m];
    F.dg = dg;
    F.r = r;
    F.z = z;
    F.nlist = (int32_t)((int64_t)((g.ni - 1) / 2) * (g.nj - 2) * (g.nk - 2));
    F.list[0] = lists;
    F.pk[0] = lists + F.nlist;
    F.list[1] = lists + 2 * (int64_t)F.nlist;
    F.pk[1] = lists + 3 * (int64_t)F.nlist;
    int round = 0, nr, conv = 0, inner = 0, fallback = 0;
    double norm = 0;
    /* linear mode (lin_y != null): Newton on F(y) = J y - b with J frozen at
     * phi solves J y = b; the stopping test is relative to the first update */
    const bool linear = lin_y != nullptr;
    /* float inner solve of the nonlinear problem: the Newton residual and
     * update run in double-float arithmetic on the float pipes (the float64
     * pipe of this GPU is narrow) from phi and rho / eps0 split once into
     * (hi, lo) pairs here; phi is rebuilt from its pairs after the last
     * update */
    const bool dfm = sizeof(T) == sizeof(float) && !linear && dfbuf != nullptr;
    float2 *phf = dfbuf, *rhf = dfbuf ? dfbuf + nn : nullptr;
    const dfl d_phi0 = df_of(phi0), d_inv_te0 = df_of(inv_te0), d_A0 = df_of(A0), d_inv_eps0 = df_of(inv_eps0);
    if (dfm) {
        df_prepass(phi, rho, phf, rhf, code, phi_prev, predict, d_inv_eps0, nn, gtid, gsize);
        grid.sync();
    }
    const float cl[3] = {(float)(cd[0] - (double)ct[0]), (float)(cd[1] - (double)ct[1]),
                         (float)(cd[2] - (double)ct[2])};
    double nr_scale = linear ? 0.0 : 1.0;
    double zz_stop = nr_tol * nr_tol / 4.0 * (double)nn * nr_scale;
    for (nr = 0; nr < nr_max; nr++) {
        /* Newton residual (float64) and the Boltzmann part of the Jacobian
         * diagonal; the first red smoothing half sweep (or Jacobi) of the
         * preconditioner rides along */
        double ff = 0;
        const double *XR = linear ? lin_y : phi;
        if (dfm) {
            /* the residual of the float-inner form below, in double-float:
             * per axis c (2 x_u - x_w - x_e) (a missing link reads x_u), the
             * Boltzmann factor as expf of the leading part times a
             * first-order factor for the rest, rho / eps0 from its pair */
            const float ffs = df_residual<T>(code, phf, rhf, z, dg, r, y, nn, gtid, gsize, (int32_t)sy, (int32_t)sz,
                                             ct, cl, d_phi0, d_inv_te0, d_A0, (float)A0_te0, jacobi);
            ff = (double)ffs;
        } else
        /* two nodes per pass, every load before any store; the loads do not
         * wait for the code word (neighbour indices are clamped into the
         * grid, a node past the end reads the interior node (1,1,1)), and
         * a node that is not an unknown stores nothing */
        for (int64_t u0 = gtid; u0 < nn; u0 += 2 * gsize) {
            const int64_t uq[2] = {u0, u0 + gsize};
            bool onq[2];
            uint16_t c[2];
            int64_t u[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                c[h] = uq[h] < nn ? code[uq[h]] : (uint16_t)0;
                onq[h] = c[h] & SELF;
                u[h] = uq[h] < nn ? uq[h] : safe;
            }
            double xu[2], pn[2][6], ph[2], bv[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                xu[h] = XR[u[h]];
#pragma unroll
                for (int m = 0; m < 6; m++) pn[h][m] = XR[clamp_node(u[h] + off[m], nn)];
                ph[h] = phi[u[h]];
                bv[h] = linear ? lin_b[u[h]] : rho[u[h]];
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (!onq[h]) continue;
                double Fv;
                T rv, dBt;
                if (sizeof(T) == sizeof(float)) {
                    /* the float-inner form spends fewer float64 operations
                     * (the float64 pipe is narrow here): per axis
                     * c (2 x_u - x_w - x_e) with a missing link reading x_u
                     * itself; the Boltzmann factor as the float exponential of
                     * the leading part of the argument times a first-order
                     * factor for the rest (relative error ~1e-7, which moves
                     * phi by ~Te 1e-7, far below the Newton tolerance); the
                     * Jacobian's Boltzmann diagonal in float */
                    double L = 0;
#pragma unroll
                    for (int a = 0; a < 3; a++) {
                        const unsigned mw = (1u << (2 * a)) | (1u << (6 + 2 * a));
                        const unsigned me = (1u << (2 * a + 1)) | (1u << (7 + 2 * a));
                        const double pw = (c[h] & mw) ? pn[h][2 * a] : xu[h];
                        const double pe = (c[h] & me) ? pn[h][2 * a + 1] : xu[h];
                        L = fma(cd[a], fma(2.0, xu[h], -(pw + pe)), L);
                    }
                    const double xa = (ph[h] - phi0) * inv_te0;
                    const float xh = (float)xa;
                    const float ef = expf(xh);
                    const double e = fma((double)ef, xa - (double)xh, (double)ef);
                    if (linear) {
                        const double dB = A0_te0 * e;
                        Fv = fma(dB, xu[h], L) - bv[h];
                        dBt = (T)dB;
                    } else {
                        Fv = fma(-bv[h], inv_eps0, fma(A0, e, L));
                        dBt = (T)((float)A0_te0 * ef);
                    }
                    rv = (T)Fv;
                    if (jacobi || !(c[h] & BLACK)) z[u[h]] = rv / full_diag(c[h], dBt, ct);
                } else {
                    double L = 0, dL = 0;
#pragma unroll
                    for (int m = 0; m < 6; m++) {
                        const bool on = c[h] & ((1u << m) | (1u << (6 + m)));
                        L += on ? cd[m >> 1] * (xu[h] - pn[h][m]) : 0.0;
                        dL += on ? cd[m >> 1] : 0.0;
                    }
                    const double e = exp((ph[h] - phi0) * inv_te0);
                    const double dB = A0_te0 * e;
                    Fv = linear ? L + dB * xu[h] - bv[h] : L + A0 * e - bv[h] * inv_eps0;
                    rv = (T)Fv;
                    dBt = (T)dB;
                    if (jacobi || !(c[h] & BLACK)) z[u[h]] = rv / (T)(dL + dB);
                }
                dg[u[h]] = dBt;
                r[u[h]] = rv;
                y[u[h]] = 0;
                ff += Fv * Fv;
            }
        }
        double s1[1] = {ff};
        grid_sum_n<1>(grid, s1, partials, round);
        double FF = s1[0];
        if (!isfinite(FF)) {
            if (gtid == 0) atomicOr(err, DERR_NONFINITE);
            break;
        }
        bool take_z = false;
        if (FF > 0) {
            const double stop2 = pcg_tol * pcg_tol * FF;
            double ZZ;
            double RZ = vcycle_rest(grid, F, mg, partials, round, ZZ, SB);
            /* the first preconditioned residual already estimates an update
             * below the inner stop: it is the update */
            take_z = ZZ < zz_stop;
            bool inner_ok = take_z;
            T beta = 0;
            T *pold = p0, *pnew = p1;
            for (int it = 0; it < pcg_max && !take_z; it++) {
                /* p = z + beta p (on the fly at the node and its neighbours),
                 * q = J p */
                T pq = 0;
                /* two nodes per pass, every load before any store; the loads
                 * do not wait for the code word (neighbour indices clamped
                 * into the grid, a node past the end reads the interior node
                 * (1,1,1)); a node that is not an unknown stores nothing */
                for (int64_t u0 = gtid; u0 < nn; u0 += 2 * gsize) {
                    const int64_t uq[2] = {u0, u0 + gsize};
                    bool on[2];
                    uint16_t c[2];
                    int64_t u[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        c[h] = uq[h] < nn ? code[uq[h]] : (uint16_t)0;
                        on[h] = c[h] & SELF;
                        u[h] = uq[h] < nn ? uq[h] : safe;
                    }
                    /* an unknown is interior: neighbour loads need no code bit */
                    T zc[2], pc[2], dB[2], zn[2][6], pn[2][6];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        zc[h] = z[u[h]];
                        pc[h] = it ? pold[u[h]] : (T)0;
                        dB[h] = dg[u[h]];
#pragma unroll
                        for (int m = 0; m < 6; m++) {
                            const int64_t nb = clamp_node(u[h] + off[m], nn);
                            zn[h][m] = z[nb];
                            pn[h][m] = it ? pold[nb] : (T)0;
                        }
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (!on[h]) continue;
                        T pu = zc[h] + beta * pc[h];
#pragma unroll
                        for (int m = 0; m < 6; m++) pn[h][m] = zn[h][m] + beta * pn[h][m];
                        T s = jacobian_apply(c[h], dB[h], ct, pu, pn[h]);
                        pnew[u[h]] = pu;
                        q[u[h]] = s;
                        pq += pu * s;
                    }
                }
                const T t3[1] = {pq};
                double s3[1];
                grid_sum_t<1, T>(grid, t3, s3, partials, round);
                /* block-uniform scalars are computed by one thread and
                 * broadcast: 32 warps each dividing in float64 would queue
                 * on the narrow float64 pipe */
                if (threadIdx.x == 0) bc_alpha = (T)(RZ / s3[0]);
                __syncthreads();
                const T alpha = bc_alpha;
                /* y += alpha p, r -= alpha q, and the first red half sweep */
                T rr = 0;
                for (int64_t u0 = gtid; u0 < nn; u0 += 2 * gsize) {
                    const int64_t uq[2] = {u0, u0 + gsize};
                    bool on[2];
                    uint16_t c[2];
                    int64_t u[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        c[h] = uq[h] < nn ? code[uq[h]] : (uint16_t)0;
                        on[h] = c[h] & SELF;
                        u[h] = uq[h] < nn ? uq[h] : safe;
                    }
                    T yv[2], pv[2], rv[2], qv[2], dv[2];
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        yv[h] = y[u[h]];
                        pv[h] = pnew[u[h]];
                        rv[h] = r[u[h]];
                        qv[h] = q[u[h]];
                        dv[h] = dg[u[h]];
                    }
#pragma unroll
                    for (int h = 0; h < 2; h++) {
                        if (!on[h]) continue;
                        y[u[h]] = yv[h] + alpha * pv[h];
                        T ru = rv[h] - alpha * qv[h];
                        r[u[h]] = ru;
                        rr += ru * ru;
                        if (jacobi || !(c[h] & BLACK)) z[u[h]] = ru / full_diag(c[h], dv[h], ct);
                    }
                }
                const T t4[1] = {rr};
                double s4[1];
                grid_sum_t<1, T>(grid, t4, s4, partials, round);
                inner++;
                if (threadIdx.x == 0) bc_stop = !(s4[0] > stop2); /* also leaves on NaN */
                __syncthreads();
                if (bc_stop) {
                    inner_ok = true;
                    break;
                }
                double RZn = vcycle_rest(grid, F, mg, partials, round, ZZ, SB);
                /* z = M r estimates the remaining error of y: once its RMS is
                 * below half the Newton tolerance, further inner
                 * iterations cannot change the outcome of the Newton test */
                if (threadIdx.x == 0) {
                    bc_stop = ZZ < zz_stop;
                    bc_beta = (T)(RZn / RZ);
                }
                __syncthreads();
                if (bc_stop) {
                    inner_ok = true;
                    break;
                }
                beta = bc_beta;
                RZ = RZn;
                T *tp = pold;
                pold = pnew;
                pnew = tp;
            }
            /* The reference's fallback when the linear PCG fails
             * (ch3/ver2/PotentialSolver.cpp:270-271, solveGSLinear :433-461):
             * Gauss-Seidel (omega 1) on the same linear system from the
             * inner solve's last iterate, the residual's RMS checked every
             * 25 sweeps (from the first) against the solver tolerance, at
             * most gs_max sweeps.  Here the sweeps are red-black and act on
             * the correction, J e = r from e = 0 (r = F - J y is the PCG's
             * residual), then y += e. */
            if (!inner_ok && gs_max > 0) {
                for (int64_t u = gtid; u < nn; u += gsize) z[u] = (T)0;
                grid.sync();
                for (int sw = 0; sw < gs_max; sw++) {
                    for (int col = 0; col < 2; col++) {
                        for (int64_t u = gtid; u < nn; u += gsize) {
                            const uint16_t cc = code[u];
                            if (!(cc & SELF) || ((cc & BLACK) ? 1 : 0) != col) continue;
                            T acc = r[u];
#pragma unroll
                            for (int m = 0; m < 6; m++)
                                if (cc & (1u << m)) acc += ct[m >> 1] * z[u + off[m]];
                            z[u] = acc / full_diag(cc, dg[u], ct);
                        }
                        grid.sync();
                    }
                    fallback++;
                    if (sw % 25 == 0) {
                        T rr2 = 0;
                        for (int64_t u = gtid; u < nn; u += gsize) {
                            const uint16_t cc = code[u];
                            if (!(cc & SELF)) continue;
                            T xn[6];
#pragma unroll
                            for (int m = 0; m < 6; m++) xn[m] = (cc & (1u << m)) ? z[u + off[m]] : (T)0;
                            const T R = r[u] - jacobian_apply(cc, dg[u], ct, z[u], xn);
                            rr2 += R * R;
                        }
                        const T t5[1] = {rr2};
                        double s5[1];
                        grid_sum_t<1, T>(grid, t5, s5, partials, round);
                        if (threadIdx.x == 0) bc_stop = sqrt(s5[0] / (double)nn) < gs_tol;
                        __syncthreads();
                        if (bc_stop) break;
                    }
                }
                for (int64_t u = gtid; u < nn; u += gsize)
                    if (code[u] & SELF) y[u] += z[u];
                grid.sync();
            }
        }
        /* Newton update */
        double yy = 0;
        double *X = linear ? lin_y : phi;
        if (dfm) {
            yy = (double)df_update<T>(code, take_z ? z : y, phf, nn, gtid, gsize);
        } else
        /* two nodes per pass, loads ahead of the code test and the stores */
        for (int64_t u0 = gtid; u0 < nn; u0 += 2 * gsize) {
            const int64_t uq[2] = {u0, u0 + gsize};
            int64_t u[2];
            uint16_t c[2];
            T yv[2];
            double xv[2];
#pragma unroll
            for (int h = 0; h < 2; h++) {
                u[h] = uq[h] < nn ? uq[h] : safe;
                c[h] = uq[h] < nn ? code[u[h]] : (uint16_t)0;
                yv[h] = take_z ? z[u[h]] : y[u[h]];
                xv[h] = X[u[h]];
            }
#pragma unroll
            for (int h = 0; h < 2; h++) {
                if (!(c[h] & SELF)) continue;
                const double yu = (double)yv[h];
                X[u[h]] = xv[h] - yu;
                yy += yu * yu;
            }
        }
        double s6[1] = {yy};
        grid_sum_n<1>(grid, s6, partials, round);
        norm = sqrt(s6[0] / (double)nn);
        if (!isfinite(norm)) {
            if (gtid == 0) atomicOr(err, DERR_NONFINITE);
            break;
        }
        if (linear && nr == 0) {
            nr_scale = norm;
            zz_stop = 0.01 * nr_tol * nr_tol * norm * norm * (double)nn;
        }
        if (norm < nr_tol * nr_scale || (linear && norm == 0.0)) {
            conv = 1;
            nr++;
            break;
        }
    }
    if (dfm) {
        df_rebuild(code, phf, phi, nn, gtid, gsize);
        grid.sync();
    }
    if (!linear) neumann_copies(target, phi, nn, gtid, gsize);
    if (gtid == 0) {
        st->converged = conv;
        st->iterations = nr;
        st->inner_iterations = inner;
        st->fallback_sweeps = fallback;
        st->residual = norm;
        st->solves += 1;
        st->outer_total += nr;
        st->inner_total += inner;
    }
}

/* Galerkin coarse operator of level l+1 from level l (deterministic gather:
 * one thread per coarse node, children and their links in a fixed order).
 * Level 0 is the node grid with the operator L (Dirichlet links kept on the
 * diagonal); the Boltzmann diagonal term is left to the fine smoother. */
template <typename T>
__global__ void k_mg_setup(Geo g, const uint16_t *__restrict__ code, MgLevel<T> Lf, MgLevel<T> C, int from_fine) {
    int64_t I = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (I >= C.n) return;
    int ci = (int)(I % C.nx);
    int cj = (int)((I / C.nx) % C.ny);
    int ck = (int)(I / ((int64_t)C.nx * C.ny));
    const double cd[3] = {1.0 / (g.dh[0] * g.dh[0]), 1.0 / (g.dh[1] * g.dh[1]), 1.0 / (g.dh[2] * g.dh[2])};
    double diag = 0, w[6] = {0, 0, 0, 0, 0, 0};
    int nx = from_fine ? g.ni : Lf.nx, ny = from_fine ? g.nj : Lf.ny, nz = from_fine ? g.nk : Lf.nz;
    int64_t offs[6] = {-1, 1, -(int64_t)nx, nx, -(int64_t)nx * ny, (int64_t)nx * ny};
    const int di[6] = {-1, 1, 0, 0, 0, 0}, dj[6] = {0, 0, -1, 1, 0, 0}, dk[6] = {0, 0, 0, 0, -1, 1};
    for (int d = 0; d < 8; d++) {
        int i = 2 * ci + (d & 1), j = 2 * cj + ((d >> 1) & 1), k = 2 * ck + (d >> 2);
        if (i >= nx || j >= ny || k >= nz) continue;
        int64_t u = ((int64_t)k * ny + j) * nx + i;
        if (from_fine) {
            uint16_t c = code[u];
            if (!(c & SELF)) continue;
            for (int m = 0; m < 6; m++)
                if (c & ((1u << m) | (1u << (6 + m)))) diag += cd[m >> 1];
            for (int m = 0; m < 6; m++) {
                if (!(c & (1u << m))) continue;
                bool inside = ((i + di[m]) >> 1) == ci && ((j + dj[m]) >> 1) == cj && ((k + dk[m]) >> 1) == ck;
                if (inside)
                    diag -= cd[m >> 1];
                else
                    w[m] += cd[m >> 1];
            }
        } else {
            double dd = (double)Lf.diag[u];
            if (dd == 0) continue;
            diag += dd;
            for (int m = 0; m < 6; m++) {
                double wm = (double)Lf.w[m * Lf.n + u];
                if (wm == 0) continue;
                bool inside = ((i + di[m]) >> 1) == ci && ((j + dj[m]) >> 1) == cj && ((k + dk[m]) >> 1) == ck;
                if (inside)
                    diag -= wm;
                else
                    w[m] += wm;
            }
        }
        (void)offs;
    }
    C.diag[I] = (T)diag;
    for (int m = 0; m < 6; m++) C.w[m * C.n + I] = (T)w[m];
}

/* The coarsest level's operator as a dense float64 matrix (A e = diag e -
 * sum_m w_m e_nb(m)); an aggregate without unknowns (diag 0) gets an
 * identity row. */
template <typename T>
__global__ void k_dense_build(MgLevel<T> L, double *M, double *diag0) {
    const int64_t n = L.n;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int64_t i = t / n, j = t - i * n;
    const double di = (double)L.diag[i];
    double v = 0;
    if (di == 0) {
        v = i == j ? 1.0 : 0.0;
    } else if (i == j) {
        v = di;
    } else if ((double)L.diag[j] != 0) {
        const int xi = (int)(i % L.nx), yi = (int)((i / L.nx) % L.ny), zi = (int)(i / ((int64_t)L.nx * L.ny));
        const int xj = (int)(j % L.nx), yj = (int)((j / L.nx) % L.ny), zj = (int)(j / ((int64_t)L.nx * L.ny));
        const int dx = xj - xi, dy = yj - yi, dz = zj - zi;
        int m = -1;
        if (dy == 0 && dz == 0 && (dx == -1 || dx == 1)) m = dx < 0 ? 0 : 1;
        if (dx == 0 && dz == 0 && (dy == -1 || dy == 1)) m = dy < 0 ? 2 : 3;
        if (dx == 0 && dy == 0 && (dz == -1 || dz == 1)) m = dz < 0 ? 4 : 5;
        if (m >= 0) v = -(double)L.w[m * n + i];
    }
    M[t] = v;
    if (i == j) diag0[i] = v;
}

/* In-place Gauss-Jordan inversion without pivoting (the operator is
 * symmetric positive definite), in one cooperative launch: for each k,
 * block 0 saves column k and scales row k by the pivot, then every thread
 * eliminates column k from the other rows.  A pivot that vanished against
 * the original diagonal (a singular operator) clears *ok. */
__global__ void __launch_bounds__(1024) k_gauss_jordan(double *M, int n, double *col,
                                                       const double *__restrict__ diag0, int *ok) {
    cg::grid_group grid = cg::this_grid();
    __shared__ double piv;
    for (int k = 0; k < n; k++) {
        if (blockIdx.x == 0) {
            if (threadIdx.x == 0) {
                piv = __ldcg(M + (int64_t)k * n + k);
                if (!(piv > 1e-9 * diag0[k])) {
                    *ok = 0;
                    piv = 1.0;
                }
            }
            for (int i = threadIdx.x; i < n; i += blockDim.x) col[i] = __ldcg(M + (int64_t)i * n + k);
            __syncthreads();
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                const double a = j == k ? 1.0 : __ldcg(M + (int64_t)k * n + j);
                M[(int64_t)k * n + j] = a / piv;
            }
        }
        grid.sync();
        for (int i = blockIdx.x; i < n; i += gridDim.x) {
            if (i == k) continue;
            const double f = __ldcg(col + i);
            double *Mi = M + (int64_t)i * n;
            for (int j = threadIdx.x; j < n; j += blockDim.x)
                Mi[j] = (j == k ? 0.0 : __ldcg(Mi + j)) - f * __ldcg(M + (int64_t)k * n + j);
        }
        grid.sync();
    }
}

/* the inverse in T, symmetrised; rows and columns of aggregates without
 * unknowns are zero */
template <typename T>
__global__ void k_dense_store(MgLevel<T> L, const double *__restrict__ M, T *out) {
    const int64_t n = L.n;
    const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n * n) return;
    const int64_t i = t / n, j = t - i * n;
    const bool live = (double)L.diag[i] != 0 && (double)L.diag[j] != 0;
    out[t] = live ? (T)(0.5 * (M[t] + M[j * n + i])) : (T)0;
}

/* ======================================================================== */
template <typename T>
static size_t mg_layout(World &w, MgArgs<T> &A, char *base) {
    size_t off = 0;
    int nx = (w.g.ni + 1) / 2, ny = (w.g.nj + 1) / 2, nz = (w.g.nk + 1) / 2;
    int nlev = 0, grid_levels = 1;
    while (nlev < MG_MAX) {
        MgLevel<T> &L = A.L[nlev];
        L.nx = nx;
        L.ny = ny;
        L.nz = nz;
        L.pad = 0;
        L.n = (int64_t)nx * ny * nz;
        size_t bytes = ((L.n * sizeof(T) + 255) / 256) * 256;
        L.diag = (T *)(base ? base + off : nullptr);
        off += bytes;
        L.w = (T *)(base ? base + off : nullptr);
        off += 6 * bytes;
        L.b = (T *)(base ? base + off : nullptr);
        off += bytes;
        L.e = (T *)(base ? base + off : nullptr);
        off += bytes;
        nlev++;
        if (L.n >= w.mg_block_nodes) grid_levels = nlev + 1;
        if (L.n <= 64 || (nx <= 2 && ny <= 2 && nz <= 2)) break;
        nx = (nx + 1) / 2;
        ny = (ny + 1) / 2;
        nz = (nz + 1) / 2;
    }
    A.nlev = w.mg_levels_max < nlev ? w.mg_levels_max : nlev;
    /* the first level with at most mg_dense_max nodes becomes the coarsest,
     * solved by its dense inverse on the whole grid (every level above it
     * runs on the whole grid too); the float64 work matrix of the inversion
     * and its column buffer follow the levels */
    A.dense = nullptr;
    A.dense_n = 0;
    if (w.mg_dense_max > 0)
        for (int i = 0; i < A.nlev; i++)
            if (A.L[i].n <= w.mg_dense_max) {
                A.nlev = i + 1;
                A.dense_n = (int)A.L[i].n;
                grid_levels = A.nlev + 1;
                break;
            }
    if (A.dense_n > 0) {
        const size_t nsq = (size_t)A.dense_n * A.dense_n;
        A.dense = (T *)(base ? base + off : nullptr);
        off += (nsq * sizeof(T) + 255) / 256 * 256;
        off += (nsq * sizeof(double) + 255) / 256 * 256 + 2 * (((size_t)A.dense_n * sizeof(double) + 255) / 256 * 256);
        A.dense_ok = (const int *)(base ? base + off : nullptr);
        off += 256;
    } else {
        A.dense_ok = nullptr;
    }
    A.grid_levels = grid_levels;
    A.nu_coarse = 2;
    A.scale = (T)w.mg_scale;
    /* block 0 works levels lblock-1 .. nlev-1 alone (lblock = min(grid
     * levels, nlev)); keep them in its shared memory when they fit */
    A.smem_from = -1;
    const int lblock = grid_levels < A.nlev ? grid_levels : A.nlev;
    if (A.nlev > 0 && A.nlev >= grid_levels) {
        size_t bytes = 0;
        for (int i = lblock - 1; i < A.nlev; i++) bytes += level_smem_bytes<T>(A.L[i].n);
        if (bytes <= PCG_SMEM_MAX) A.smem_from = lblock - 1;
    }
    return off;
}

template <typename T>
static int run_pcg(World &w) {
    /* the colour lists pack coordinates in 10 + 10 + 11 bits */
    if (w.g.ni > 1024 || w.g.nj > 1024 || w.g.nk > 2048) return (int)cudaErrorInvalidValue;
    size_t es = sizeof(T);
    size_t vec = ((w.nn * es + 255) / 256) * 256;
    size_t codeb = ((w.nn * sizeof(uint16_t) + 255) / 256) * 256;
    MgArgs<T> A;
    size_t mgb = mg_layout<T>(w, A, nullptr);
    int64_t nlist = (int64_t)((w.g.ni - 1) / 2) * (w.g.nj - 2) * (w.g.nk - 2);
    /* the colour lists are only read when the sweeps cannot enumerate their
     * nodes arithmetically (2^24 entries or more, see fine_half) */
    const bool need_lists = nlist >= (1 << 24);
    size_t listb = need_lists ? ((4 * nlist * sizeof(int32_t) + 255) / 256) * 256 : 0;
    /* float inner solves: the (hi, lo) pairs of phi and rho / eps0 */
    size_t dfb = sizeof(T) == sizeof(float) ? 2 * (((size_t)w.nn * sizeof(float2) + 255) / 256) * 256 : 0;
    size_t need = 7 * vec + codeb + mgb + listb + dfb;
    if (w.pcg_bytes < need || w.pcg_elem != (int)es) {
        if (w.pcg_buf) {
            cudaStreamSynchronize(w.stream);
            cudaFree(w.pcg_buf);
        }
        w.pcg_buf = nullptr;
        w.pcg_bytes = 0;
        if (cudaMalloc(&w.pcg_buf, need) != cudaSuccess) return (int)cudaErrorMemoryAllocation;
        cudaMemsetAsync(w.pcg_buf, 0, need, w.stream);
        w.pcg_bytes = need;
        w.pcg_elem = (int)es;
        w.pcg_codes_valid = false;
    }
    char *base = (char *)w.pcg_buf;
    uint16_t *code = (uint16_t *)(base + 7 * vec);
    int32_t *lists = (int32_t *)(base + 7 * vec + codeb + mgb);
    mg_layout<T>(w, A, base + 7 * vec + codeb);
    if (!w.pcg_codes_valid) {
        k_pcg_codes<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.g, w.obj, code);
        w.nlaunch++;
        for (int c = 0; c < 2 && need_lists; c++) {
            k_pcg_lists<<<blocks_for(nlist, 256), 256, 0, w.stream>>>(w.g, c, lists + 2 * c * nlist,
                                                                      lists + (2 * c + 1) * nlist);
            w.nlaunch++;
        }
        for (int l = 0; l < A.nlev; l++) {
            MgLevel<T> prev = l ? A.L[l - 1] : A.L[0];
            k_mg_setup<T><<<blocks_for(A.L[l].n, 256), 256, 0, w.stream>>>(w.g, code, prev, A.L[l], l == 0);
            w.nlaunch++;
        }
        if (A.dense) {
            const int n = A.dense_n;
            const int64_t nsq = (int64_t)n * n;
            double *M = (double *)((char *)A.dense + (nsq * sizeof(T) + 255) / 256 * 256);
            double *col = (double *)((char *)M + (nsq * sizeof(double) + 255) / 256 * 256);
            double *diag0 = col + ((size_t)n * sizeof(double) + 255) / 256 * 256 / sizeof(double);
            int *ok = (int *)A.dense_ok;
            const int one = 1;
            cudaMemcpyAsync(ok, &one, sizeof(int), cudaMemcpyHostToDevice, w.stream);
            const MgLevel<T> &Lc = A.L[A.nlev - 1];
            k_dense_build<T><<<blocks_for(nsq, 256), 256, 0, w.stream>>>(Lc, M, diag0);
            int gj_per_sm = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gj_per_sm, k_gauss_jordan, 1024, 0);
            int gj_grid = (gj_per_sm < 1 ? 1 : gj_per_sm) * w.sm_count;
            if (gj_grid > n) gj_grid = n;
            int nn_ = n;
            void *gj_args[] = {&M, &nn_, &col, &diag0, &ok};
            cudaLaunchCooperativeKernel((const void *)k_gauss_jordan, gj_grid, 1024, gj_args, 0, w.stream);
            k_dense_store<T><<<blocks_for(nsq, 256), 256, 0, w.stream>>>(Lc, M, A.dense);
            w.nlaunch += 3;
        }
        w.pcg_codes_valid = true;
    }
    const void *fn = (const void *)k_newton_pcg<T>;
    const int threads = PCG_THREADS;
    size_t dyn = 0;
    if (A.smem_from >= 0)
        for (int i = A.smem_from; i < A.nlev; i++) dyn += level_smem_bytes<T>(A.L[i].n);
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, dyn);
    if (per_sm < 1) per_sm = 1;
    int64_t maxb = (int64_t)per_sm * w.sm_count;
    int64_t needb = (w.nn + threads - 1) / threads;
    int grid = (int)(needb < maxb ? needb : maxb);
    if (grid > w.partial_slots / 4) grid = w.partial_slots / 4;
    if (w.solver_blocks > 0 && grid > w.solver_blocks) grid = w.solver_blocks;
    Geo g = w.g;
    double *phi = w.phi;
    const double *rho = w.rho;
    const int32_t *tg = w.target;
    const uint16_t *cc = code;
    double phi0 = w.phi0, te0 = w.te0, n0 = w.n0, nr_tol = w.nr_tol, pcg_tol = w.pcg_tol;
    int nr_max = w.nr_max, pcg_max = w.pcg_max;
    T *v[7];
    for (int i = 0; i < 7; i++) v[i] = (T *)(base + i * vec);
    double *part = w.d_partials;
    SolveStatus *st = w.d_status;
    int *err = w.d_err;
    const int32_t *lst = lists;
    double *ly = w.lin_y;
    const double *lb = w.lin_b;
    int gs_max = w.gs_fallback ? w.max_it : 0;
    double gs_tol = w.tol;
    /* the pairs hold nn float2 each, the second array 256-byte aligned */
    float2 *dfp = dfb ? (float2 *)(base + 7 * vec + codeb + mgb + listb) : nullptr;
    /* the predictor rides on the pairs' pass (the caller skipped k_predict) */
    double *pp = w.phi_prev;
    int predict = dfp && !ly ? w.predict_mode : 0;
    w.predict_mode = 0;
    /* the axis coefficients 1 / dh^2 rounded to T, as the kernel's cd */
    Coef3<T> ctp;
    for (int a = 0; a < 3; a++) ctp.c[a] = (T)(1.0 / (g.dh[a] * g.dh[a]));
    void *args[] = {&g,    &phi,  &rho,  &cc,   &tg,   &phi0, &te0, &n0,  &nr_max, &nr_tol, &pcg_max, &pcg_tol,
                    &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6], &A,  &lst,   &part,   &st,      &err,
                    &ly,   &lb,   &gs_max, &gs_tol, &dfp,  &pp,   &predict, &ctp};
    w.nlaunch++;
    return (int)cudaLaunchCooperativeKernel(fn, grid, threads, args, dyn, w.stream);
}

int launch_newton_pcg(World &w, bool fp32) { return fp32 ? run_pcg<float>(w) : run_pcg<double>(w); }

/* y = J^-1 b on the unknowns, J the Jacobian of the Boltzmann problem at the
 * current phi (the adjoint solve: J is symmetric); y must be zero off the
 * unknowns.  Outer iterations until the update's RMS is below rel_tol times
 * the first one's. */
int launch_pcg_linear(World &w, bool fp32, const double *b, double *y, double rel_tol, int max_outer) {
    double keep_tol = w.nr_tol;
    int keep_max = w.nr_max;
    w.lin_b = b;
    w.lin_y = y;
    w.nr_tol = rel_tol;
    w.nr_max = max_outer;
    int rc = fp32 ? run_pcg<float>(w) : run_pcg<double>(w);
    w.lin_b = nullptr;
    w.lin_y = nullptr;
    w.nr_tol = keep_tol;
    w.nr_max = keep_max;
    return rc;
}

}  // namespace espic
