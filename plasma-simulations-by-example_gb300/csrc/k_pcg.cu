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
 * order, so every block takes the same branch.
 */
#include <cooperative_groups.h>

#include "espic_world.h"

namespace cg = cooperative_groups;

namespace espic {

#define PCG_EPS_0 8.85418782e-12
#define PCG_QE 1.602176565e-19

enum : uint16_t { SELF = 1u << 12 };

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
    if (threadIdx.x < NV) {
        double s = 0;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) s += sh[threadIdx.x][k];
        slot[(size_t)blockIdx.x * NV + threadIdx.x] = s;
    }
    round++;
    grid.sync();
    if (threadIdx.x < NV) {
        double s = 0;
        for (unsigned b = 0; b < gridDim.x; b++) s += slot[(size_t)b * NV + threadIdx.x];
        tot[threadIdx.x] = s;
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < NV; q++) v[q] = tot[q];
}

template <typename T>
__global__ void __launch_bounds__(256) k_newton_pcg(Geo g, double *phi, const double *__restrict__ rho,
                                                    const uint16_t *__restrict__ code,
                                                    const int32_t *__restrict__ target, double phi0, double te0,
                                                    double n0, int nr_max, double nr_tol, int pcg_max,
                                                    double pcg_tol, T *y, T *r, T *z, T *p, T *q, T *dg,
                                                    double *partials, SolveStatus *st, int *err) {
    cg::grid_group grid = cg::this_grid();
    const int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    const int64_t off[6] = {-1, 1, -sy, sy, -sz, sz};
    const double cd[3] = {1.0 / (g.dh[0] * g.dh[0]), 1.0 / (g.dh[1] * g.dh[1]), 1.0 / (g.dh[2] * g.dh[2])};
    const T ct[3] = {(T)cd[0], (T)cd[1], (T)cd[2]};
    const double A0 = PCG_QE * n0 / PCG_EPS_0;
    const int64_t gtid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t gsize = (int64_t)gridDim.x * blockDim.x;
    int round = 0, nr, conv = 0, inner = 0;
    double norm = 0;
    for (nr = 0; nr < nr_max; nr++) {
        /* Newton residual and Jacobian diagonal (float64) */
        T ff = 0, rz = 0;
        for (int64_t u = gtid; u < nn; u += gsize) {
            uint16_t c = code[u];
            if (!(c & SELF)) continue;
            double ph = phi[u], L = 0, dL = 0;
#pragma unroll
            for (int m = 0; m < 6; m++) {
                if (c & ((1u << m) | (1u << (6 + m)))) {
                    L += cd[m >> 1] * (ph - phi[u + off[m]]);
                    dL += cd[m >> 1];
                }
            }
            double e = exp((ph - phi0) / te0);
            double F = L + A0 * e - rho[u] / PCG_EPS_0;
            T d = (T)(dL + A0 / te0 * e);
            T rr = (T)F;
            T zz = rr / d;
            dg[u] = d;
            r[u] = rr;
            z[u] = zz;
            p[u] = zz;
            y[u] = 0;
            ff += (T)(F * F);
            rz += rr * zz;
        }
        double s2[2] = {(double)ff, (double)rz};
        grid_sum_n<2>(grid, s2, partials, round);
        double FF = s2[0], RZ = s2[1];
        if (!isfinite(FF)) {
            if (gtid == 0) atomicOr(err, DERR_NONFINITE);
            break;
        }
        if (FF > 0) {
            const double stop2 = pcg_tol * pcg_tol * FF;
            for (int it = 0; it < pcg_max; it++) {
                T pq = 0;
                for (int64_t u = gtid; u < nn; u += gsize) {
                    uint16_t c = code[u];
                    if (!(c & SELF)) continue;
                    T pu = p[u];
                    T s = dg[u] * pu;
#pragma unroll
                    for (int m = 0; m < 6; m++)
                        if (c & (1u << m)) s -= ct[m >> 1] * p[u + off[m]];
                    q[u] = s;
                    pq += pu * s;
                }
                double s1[1] = {(double)pq};
                grid_sum_n<1>(grid, s1, partials, round);
                const T alpha = (T)(RZ / s1[0]);
                T rr = 0, rzn = 0;
                for (int64_t u = gtid; u < nn; u += gsize) {
                    if (!(code[u] & SELF)) continue;
                    T yy = y[u] + alpha * p[u];
                    T ru = r[u] - alpha * q[u];
                    T zu = ru / dg[u];
                    y[u] = yy;
                    r[u] = ru;
                    z[u] = zu;
                    rr += ru * ru;
                    rzn += ru * zu;
                }
                double s3[2] = {(double)rr, (double)rzn};
                grid_sum_n<2>(grid, s3, partials, round);
                inner++;
                if (!(s3[0] > stop2)) break; /* also leaves on NaN */
                const T beta = (T)(s3[1] / RZ);
                RZ = s3[1];
                for (int64_t u = gtid; u < nn; u += gsize) {
                    if (!(code[u] & SELF)) continue;
                    p[u] = z[u] + beta * p[u];
                }
                grid.sync();
            }
        }
        /* Newton update */
        T yy = 0;
        for (int64_t u = gtid; u < nn; u += gsize) {
            if (!(code[u] & SELF)) continue;
            T yu = y[u];
            phi[u] -= (double)yu;
            yy += yu * yu;
        }
        double s4[1] = {(double)yy};
        grid_sum_n<1>(grid, s4, partials, round);
        norm = sqrt(s4[0] / (double)nn);
        if (!isfinite(norm)) {
            if (gtid == 0) atomicOr(err, DERR_NONFINITE);
            break;
        }
        if (norm < nr_tol) {
            conv = 1;
            nr++;
            break;
        }
    }
    /* Neumann boundary nodes take the value at the end of their chain */
    for (int64_t u = gtid; u < nn; u += gsize) {
        int32_t t = target[u];
        if (t >= 0) phi[u] = phi[t];
    }
    if (gtid == 0) {
        st->converged = conv;
        st->iterations = nr;
        st->inner_iterations = inner;
        st->residual = norm;
        st->solves += 1;
        st->outer_total += nr;
        st->inner_total += inner;
    }
}

/* ======================================================================== */
struct PcgBufs {
    uint16_t *code;
    void *v[6];
};

static bool pcg_alloc(World &w, bool fp32) {
    size_t es = fp32 ? sizeof(float) : sizeof(double);
    size_t vec = ((w.nn * es + 255) / 256) * 256;
    size_t need = 6 * vec + ((w.nn * sizeof(uint16_t) + 255) / 256) * 256;
    if (w.pcg_bytes < need) {
        if (w.pcg_buf) cudaFree(w.pcg_buf);
        w.pcg_buf = nullptr;
        w.pcg_bytes = 0;
        if (cudaMalloc(&w.pcg_buf, need) != cudaSuccess) return false;
        w.pcg_bytes = need;
        w.pcg_codes_valid = false;
    }
    return true;
}

int launch_newton_pcg(World &w, bool fp32) {
    if (!pcg_alloc(w, fp32)) return (int)cudaErrorMemoryAllocation;
    size_t es = fp32 ? sizeof(float) : sizeof(double);
    size_t vec = ((w.nn * es + 255) / 256) * 256;
    char *base = (char *)w.pcg_buf;
    uint16_t *code = (uint16_t *)(base + 6 * vec);
    if (!w.pcg_codes_valid) {
        k_pcg_codes<<<blocks_for(w.nn, 256), 256, 0, w.stream>>>(w.g, w.obj, code);
        w.nlaunch++;
        w.pcg_codes_valid = true;
    }
    const void *fn = fp32 ? (const void *)k_newton_pcg<float> : (const void *)k_newton_pcg<double>;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, 0);
    if (per_sm < 1) per_sm = 1;
    int64_t maxb = (int64_t)per_sm * w.sm_count;
    int64_t need = (w.nn + 255) / 256;
    int grid = (int)(need < maxb ? need : maxb);
    if (grid > w.partial_slots / 4) grid = w.partial_slots / 4;
    Geo g = w.g;
    double *phi = w.phi;
    const double *rho = w.rho;
    const int32_t *tg = w.target;
    const uint16_t *cc = code;
    double phi0 = w.phi0, te0 = w.te0, n0 = w.n0, nr_tol = w.nr_tol, pcg_tol = w.pcg_tol;
    int nr_max = w.nr_max, pcg_max = w.pcg_max;
    void *v[6];
    for (int i = 0; i < 6; i++) v[i] = base + i * vec;
    double *part = w.d_partials;
    SolveStatus *st = w.d_status;
    int *err = w.d_err;
    void *args[] = {&g,      &phi,     &rho,  &cc,   &tg,   &phi0, &te0,  &n0,   &nr_max, &nr_tol, &pcg_max,
                    &pcg_tol, &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &part, &st,    &err};
    w.nlaunch++;
    return (int)cudaLaunchCooperativeKernel(fn, grid, 256, args, 0, w.stream);
}

}  // namespace espic
