/*
 * k_ensemble.cu -- a batched ensemble of independent grounded boxes (the ch2
 * box of ch2/Main.cpp:14-75, one per ensemble member) stepped together on one
 * GPU.  Boxes differ in node counts, particle counts, species weights and
 * densities.  Compiled with -fmad=false: the float64 density, charge and E
 * arithmetic is the one of k_fp64.cu (World::computeChargeDensity,
 * ch2/World.cpp:46-54; PotentialSolver::computeEF, ch2/PotentialSolver.cpp:
 * 70-110), so a box of the ensemble reproduces the same box run as a World.
 *
 * Layout in HBM: node fields of all boxes concatenated (box b owns nodes
 * [node0_b, node0_b + nn_b)): phi, rho (f64), ef4 (float4), the SOR
 * correction and residual (f32), and one int64 fixed-point accumulator per
 * species; particles of all (box, species) segments concatenated in the
 * mixed form (cell key, f32 offsets, f32 velocity), each segment starting on
 * a 64-particle boundary.
 *
 * A step is two persistent launches, captured once in a CUDA graph:
 *  1. k_ens_push (k_mixed.cu): push + deposit over a flattened work list of
 *     particle chunks; the walls reflect, so counts never change and the
 *     work list is built once on the host;
 *  2. k_ens_solve: thread-block clusters (1 to 8 CTAs on as many SMs) claim
 *     boxes, largest first, from an atomic counter; per box: rho from the
 *     accumulators (which it clears), the red-black SOR of
 *     PotentialSolver::solve (ch2/PotentialSolver.cpp:11-67) as float32
 *     correction sweeps under a float64 residual, then E, every pass split
 *     over the cluster's CTAs between cluster barriers.
 *
 * The SOR: the residual R = rho/eps0 + L phi of the reference
 * (ch2/PotentialSolver.cpp:44-61, L2 = sqrt(sum R^2 / (ni nj nk))) is formed
 * in float64; while L2 >= tol, 25 red-black sweeps solve L e = -R for a
 * float32 correction e (e = 0 on the walls) and phi += e.  The float64
 * residual bounds the error of phi, the float32 sweeps do the work.  Its
 * reduction uses a fixed virtual width of 1024 partial sums and a fixed tree,
 * so results do not depend on the block size the autotuner picks.
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include <cooperative_groups.h>

#include "espic.h"
#include "espic_world.h"

namespace cg = cooperative_groups;

int espic_internal_fail(int code, const char *msg);

namespace espic {

#define ENS_EPS_0 8.85418782e-12
constexpr int ENS_VW = 1024;      /* virtual width of the deterministic reductions */
constexpr int ENS_SWEEPS = 25;    /* float32 sweeps between float64 residual checks */

/* a / b correctly rounded, given y = RN(1/b) for b > 0: q = a y, the exact
 * remainder r = a - b q (one FMA) and q + r y rounded, Markstein's
 * correction (P. Markstein, IBM J. Res. Develop. 34(1), 1990), which yields
 * the correctly rounded quotient for normal operands; a = +-0 returns a y,
 * the zero of the right sign.  Three float64 operations instead of a
 * division, whose cost the GB300's float64 rate makes dominant. */
__device__ __forceinline__ double div_rcp(double a, double b, double y) {
    const double q = a * y;
    const double r = __fma_rn(-q, b, a);
    const double q2 = __fma_rn(r, y, q);
    /* a == +-0 tested on the bits: an integer compare keeps the narrow
     * float64 pipe for the arithmetic */
    return zero_bits(a) ? q : q2;
}

/* sum of part[0..ENS_VW) in a fixed tree; every thread gets the total */
__device__ double ens_tree_sum(double *part) {
    __syncthreads();
    for (int w = ENS_VW / 2; w > 0; w >>= 1) {
        for (int v = threadIdx.x; v < w; v += blockDim.x) part[v] += part[v + w];
        __syncthreads();
    }
    double t = part[0];
    __syncthreads();
    return t;
}

__device__ __forceinline__ double ens_node_volume(const Geo &g, int i, int j, int k) {
    double V = g.dh[0] * g.dh[1] * g.dh[2];
    if (i == 0 || i == g.ni - 1) V *= 0.5;
    if (j == 0 || j == g.nj - 1) V *= 0.5;
    if (k == 0 || k == g.nk - 1) V *= 0.5;
    return V;
}

/* d / node_vol: node_vol = V0 2^-h (h boundary halvings), so the quotient is
 * the correctly rounded d / V0 scaled by 2^h, exactly */
__device__ __forceinline__ double ens_per_volume(const Geo &g, int i, int j, int k, double d, double V0,
                                                 double yV0) {
    double scale = 1.0;
    if (i == 0 || i == g.ni - 1) scale *= 2.0;
    if (j == 0 || j == g.nj - 1) scale *= 2.0;
    if (k == 0 || k == g.nk - 1) scale *= 2.0;
    return div_rcp(d, V0, yV0) * scale;
}

/* reciprocals of 2 dh per axis: the divisors of the E differences */
struct EfRcp {
    double d2[3], y2[3];
};

__device__ __forceinline__ EfRcp ef_rcp(const Geo &g) {
    EfRcp r;
    for (int d = 0; d < 3; d++) {
        r.d2[d] = 2 * g.dh[d];
        r.y2[d] = 1.0 / r.d2[d];
    }
    return r;
}

/* E at node u = (i, j, k) of a box, the differences of k_efield (the same
 * numerators; the division by 2 dh correctly rounded through div_rcp) */
__device__ __forceinline__ void ens_efield(const Geo &g, const EfRcp &rc, const double *phi, int64_t u, int i, int j,
                                           int k, double &e0, double &e1, double &e2) {
    const int64_t sy = g.ni, sz = (int64_t)g.ni * g.nj;
    double n0, n1, n2;
    if (i == 0)
        n0 = -(-3 * phi[u] + 4 * phi[u + 1] - phi[u + 2]);
    else if (i == g.ni - 1)
        n0 = -(phi[u - 2] - 4 * phi[u - 1] + 3 * phi[u]);
    else
        n0 = -(phi[u + 1] - phi[u - 1]);
    if (j == 0)
        n1 = -(-3 * phi[u] + 4 * phi[u + sy] - phi[u + 2 * sy]);
    else if (j == g.nj - 1)
        n1 = -(phi[u - 2 * sy] - 4 * phi[u - sy] + 3 * phi[u]);
    else
        n1 = -(phi[u + sy] - phi[u - sy]);
    if (k == 0)
        n2 = -(-3 * phi[u] + 4 * phi[u + sz] - phi[u + 2 * sz]);
    else if (k == g.nk - 1)
        n2 = -(phi[u - 2 * sz] - 4 * phi[u - sz] + 3 * phi[u]);
    else
        n2 = -(phi[u + sz] - phi[u - sz]);
    e0 = div_rcp(n0, rc.d2[0], rc.y2[0]);
    e1 = div_rcp(n1, rc.d2[1], rc.y2[1]);
    e2 = div_rcp(n2, rc.d2[2], rc.y2[2]);
}

/* cluster barrier between passes that exchange global memory across the
 * cluster's SMs: barrier.cluster.arrive (release) + wait (acquire) orders
 * every CTA's global writes before the other CTAs' later reads */
__device__ __forceinline__ void cluster_sync_global(cg::cluster_group &cl) { cl.sync(); }

/* One box per thread-block cluster of C CTAs (C = 1, 2, 4 or 8, chosen at
 * launch): the CTAs split every node pass and every half sweep into
 * contiguous slices and meet at cluster barriers.  The box a cluster works
 * on is claimed by CTA 0 and read by the others from its shared memory.  The
 * residual sum uses the fixed layout of ENS_VW virtual threads (node t
 * belongs to virtual thread t mod ENS_VW; CTA r owns a contiguous range of
 * virtual threads); CTA 0 gathers the ENS_VW partials through distributed
 * shared memory and sums them in a fixed tree, so the result depends on
 * neither C nor the block size. */
__global__ void __launch_bounds__(1024) k_ens_solve(const EnsBox *__restrict__ boxes, const EnsSeg *__restrict__ segs,
                                                    int nsp, const int *__restrict__ order, int nbox, int *counter,
                                                    double *phi, double *rho, float *ecor, float *res, float4 *ef4,
                                                    unsigned long long *acc, int64_t total_nodes, int max_it,
                                                    double tol, int solve, EnsStat *stat, int *err) {
    cg::cluster_group cl = cg::this_cluster();
    const int C = (int)cl.num_blocks();
    const int rank = (int)cl.block_rank();
    __shared__ double part[ENS_VW];
    __shared__ double total;
    __shared__ int sb;
    const int tid = threadIdx.x, nt = blockDim.x;
    const int vper = ENS_VW / C, v0 = rank * vper, v1 = v0 + vper;
    for (;;) {
        if (rank == 0 && tid == 0) sb = atomicAdd(counter, 1);
        cluster_sync_global(cl);
        const int b = *cl.map_shared_rank(&sb, 0);
        cluster_sync_global(cl);
        if (b >= nbox) break;
        const int bid = order[b];
        const EnsBox B = boxes[bid];
        const Geo g = B.g;
        const int ni = g.ni, nj = g.nj, nk = g.nk;
        const int64_t nn = B.nn;
        double *ph = phi + B.node0;
        double *rh = rho + B.node0;
        float *e = ecor + B.node0;
        float *R = res + B.node0;
        const int64_t n0 = nn * rank / C, n1 = nn * (rank + 1) / C;
        /* 1. rho = sum_s q_s den_s, den_s = counts * unit_s / node_vol; the
         *    accumulators are cleared for the next deposit */
        const double V0 = g.dh[0] * g.dh[1] * g.dh[2];
        const double yV0 = 1.0 / V0;
        for (int64_t u = n0 + tid; u < n1; u += nt) {
            const int i = (int)(u % ni), j = (int)((u / ni) % nj), k = (int)(u / ((int64_t)ni * nj));
            double r = 0;
            for (int s = 0; s < nsp; s++) {
                const EnsSeg &sg = segs[bid * nsp + s];
                unsigned long long *A = acc + (int64_t)s * total_nodes + B.node0;
                const double d = __ll2double_rn((long long)A[u]) * sg.unit;
                const double den = ens_per_volume(g, i, j, k, d, V0, yV0);
                A[u] = 0ull;
                if (sg.q != 0) r += den * sg.q;
            }
            rh[u] = r;
            e[u] = 0.f;
        }
        cluster_sync_global(cl);
        /* 2. red-black SOR: float32 correction sweeps under the float64
         *    residual */
        const double idx2 = 1.0 / (g.dh[0] * g.dh[0]);
        const double idy2 = 1.0 / (g.dh[1] * g.dh[1]);
        const double idz2 = 1.0 / (g.dh[2] * g.dh[2]);
        const double D = 2 * idx2 + 2 * idy2 + 2 * idz2;
        const float fcx = (float)idx2, fcy = (float)idy2, fcz = (float)idz2, fiD = (float)(1.0 / D);
        const double yeps = 1.0 / ENS_EPS_0;
        const float fw = (float)B.omega;
        const int sy = ni, sz = ni * nj;
        const int hx = (ni - 2 + 1) / 2;
        const int count = hx * (nj - 2) * (nk - 2);
        const int interior = (ni - 2) * (nj - 2) * (nk - 2);
        const int c0 = (int)((int64_t)count * rank / C), c1 = (int)((int64_t)count * (rank + 1) / C);
        const int i0 = (int)((int64_t)interior * rank / C), i1 = (int)((int64_t)interior * (rank + 1) / C);
        int sweeps = 0, conv = 0;
        double L2 = 0;
        while (solve) {
            for (int v = v0 + tid; v < v1; v += nt) {
                double acc2 = 0;
                for (int t = v; t < interior; t += ENS_VW) {
                    const int i = 1 + t % (ni - 2);
                    const int r = t / (ni - 2);
                    const int j = 1 + r % (nj - 2);
                    const int k = 1 + r / (nj - 2);
                    const int u = (k * nj + j) * ni + i;
                    const double Ru = -ph[u] * D + div_rcp(rh[u], ENS_EPS_0, yeps) + idx2 * (ph[u - 1] + ph[u + 1]) +
                                      idy2 * (ph[u - sy] + ph[u + sy]) + idz2 * (ph[u - sz] + ph[u + sz]);
                    R[u] = (float)Ru;
                    e[u] = 0.f;
                    acc2 += Ru * Ru;
                }
                part[v] = acc2;
            }
            cluster_sync_global(cl);
            if (rank == 0) {
                for (int v = vper + tid; v < ENS_VW; v += nt) part[v] = *cl.map_shared_rank(&part[v], v / vper);
                const double t = ens_tree_sum(part);
                if (tid == 0) total = t;
            }
            cluster_sync_global(cl);
            L2 = sqrt(*cl.map_shared_rank(&total, 0) / ((double)ni * nj * nk));
            if (!isfinite(L2)) {
                if (rank == 0 && tid == 0) atomicOr(err, DERR_NONFINITE);
                break;
            }
            if (L2 < tol) {
                conv = 1;
                break;
            }
            if (sweeps >= max_it) break;
            /* ENS_SWEEPS float32 sweeps of L e = -R, then phi += e and the
             * float64 residual decides again */
            const int ns = max_it - sweeps < ENS_SWEEPS ? max_it - sweeps : ENS_SWEEPS;
            for (int s = 0; s < ns; s++) {
                for (int c = 0; c < 2; c++) {
                    /* four independent nodes of colour c per thread: all
                     * loads before any store */
                    for (int tb = c0 + tid; tb < c1; tb += 4 * nt) {
                        int uq[4];
                        float eo[4], sum[4];
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            const int t = tb + q * nt;
                            uq[q] = -1;
                            eo[q] = 0.f;
                            sum[q] = 0.f;
                            if (t >= c1) continue;
                            const int i2 = t % hx;
                            const int r = t / hx;
                            const int j = 1 + r % (nj - 2);
                            const int k = 1 + r / (nj - 2);
                            const int i = 1 + 2 * i2 + ((1 + j + k + c) & 1);
                            if (i > ni - 2) continue;
                            const int u = (k * nj + j) * ni + i;
                            uq[q] = u;
                            eo[q] = e[u];
                            sum[q] = R[u] + fcx * (e[u - 1] + e[u + 1]) + fcy * (e[u - sy] + e[u + sy]) +
                                     fcz * (e[u - sz] + e[u + sz]);
                        }
#pragma unroll
                        for (int q = 0; q < 4; q++) {
                            if (uq[q] < 0) continue;
                            const float en = sum[q] * fiD;
                            e[uq[q]] = eo[q] + fw * (en - eo[q]);
                        }
                    }
                    cluster_sync_global(cl);
                }
            }
            sweeps += ns;
            for (int t = i0 + tid; t < i1; t += nt) {
                const int i = 1 + t % (ni - 2);
                const int r = t / (ni - 2);
                const int j = 1 + r % (nj - 2);
                const int k = 1 + r / (nj - 2);
                const int u = (k * nj + j) * ni + i;
                ph[u] += (double)e[u];
            }
            cluster_sync_global(cl);
        }
        /* 3. E = -grad phi, float32 copy for the push */
        const EfRcp rc = ef_rcp(g);
        for (int64_t u = n0 + tid; u < n1; u += nt) {
            const int i = (int)(u % ni), j = (int)((u / ni) % nj), k = (int)(u / ((int64_t)ni * nj));
            double e0, e1, e2;
            ens_efield(g, rc, ph, u, i, j, k, e0, e1, e2);
            ef4[B.node0 + u] = make_float4((float)e0, (float)e1, (float)e2, 0.f);
        }
        if (rank == 0 && tid == 0) {
            stat[bid].sweeps = sweeps;
            stat[bid].converged = conv;
            stat[bid].residual = L2;
        }
        cluster_sync_global(cl);
    }
}

/* float64 E of one box (for reading) */
__global__ void k_ens_efield64(Geo g, const double *__restrict__ phi, double *ef) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    const int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
    double e0, e1, e2;
    ens_efield(g, ef_rcp(g), phi, u, i, j, k, e0, e1, e2);
    ef[3 * u] = e0;
    ef[3 * u + 1] = e1;
    ef[3 * u + 2] = e2;
}

/* den of one species of one box from its accumulator (for reading) */
__global__ void k_ens_density(Geo g, const unsigned long long *__restrict__ acc, double unit, double *den) {
    int64_t u = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t nn = (int64_t)g.ni * g.nj * g.nk;
    if (u >= nn) return;
    const int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
    const double V0 = g.dh[0] * g.dh[1] * g.dh[2];
    const double d = __ll2double_rn((long long)acc[u]) * unit;
    den[u] = ens_per_volume(g, i, j, k, d, V0, 1.0 / V0);
}

/* loadParticlesBox (ch2/Species.cpp:74-97) into a segment: x = x1 + U (x2 -
 * x1) per axis from Philox stream `stream` (uniforms 3p, 3p+1, 3p+2), v = 0
 * (the half-step rewind of addParticle with the zero field of a new box) */
__global__ void k_ens_load(Geo g, double3 x1, double3 x2, int64_t n, uint64_t seed, uint64_t stream, int64_t first,
                           int32_t *cell, float *off, float *vel, int64_t stride) {
    int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const double a[3] = {x1.x, x1.y, x1.z}, b[3] = {x2.x, x2.y, x2.z};
    const int nmax[3] = {g.ni, g.nj, g.nk};
    int c[3];
    for (int d = 0; d < 3; d++) {
        const double x = a[d] + philox_uniform(seed, stream, 3 * (uint64_t)p + d) * (b[d] - a[d]);
        const double lc = (x - g.x0[d]) / g.dh[d];
        int i = (int)lc;
        if (i < 0) i = 0;
        if (i > nmax[d] - 2) i = nmax[d] - 2;
        c[d] = i;
        off[d * stride + first + p] = (float)(lc - i);
        vel[d * stride + first + p] = 0.f;
    }
    cell[first + p] = c[0] | (c[1] << 10) | (c[2] << 20);
}

/* per box: kinetic energy of every species (0.5 m mpw0 sum v^2, getKE of
 * ch2/Species.cpp:144-168) and the field energy 0.5 eps0 sum E^2 dV
 * (World::getPE, ch2/World.cpp:72-84); one block per box, fixed order */
__global__ void __launch_bounds__(256) k_ens_diag(const EnsBox *__restrict__ boxes, const EnsSeg *__restrict__ segs,
                                                  int nsp, const double *__restrict__ mass, const double *mpw,
                                                  const double *__restrict__ phi, const float *__restrict__ vel,
                                                  int64_t stride, double *out) {
    __shared__ double part[ENS_VW];
    const int bid = blockIdx.x;
    const EnsBox B = boxes[bid];
    const Geo g = B.g;
    const int ncol = nsp + 1;
    for (int s = 0; s < nsp; s++) {
        const EnsSeg sg = segs[bid * nsp + s];
        for (int v = threadIdx.x; v < ENS_VW; v += blockDim.x) {
            double a = 0;
            for (int64_t q = v; q < sg.n; q += ENS_VW) {
                const int64_t p = sg.p0 + q;
                const double vx = vel[p], vy = vel[stride + p], vz = vel[2 * stride + p];
                a += vx * vx + vy * vy + vz * vz;
            }
            part[v] = a;
        }
        const double t = ens_tree_sum(part);
        if (threadIdx.x == 0) out[bid * ncol + s] = 0.5 * mass[s] * mpw[bid * nsp + s] * t;
    }
    const double *ph = phi + B.node0;
    const EfRcp rc = ef_rcp(g);
    for (int v = threadIdx.x; v < ENS_VW; v += blockDim.x) {
        double a = 0;
        for (int64_t u = v; u < B.nn; u += ENS_VW) {
            const int i = (int)(u % g.ni), j = (int)((u / g.ni) % g.nj), k = (int)(u / ((int64_t)g.ni * g.nj));
            double e0, e1, e2;
            ens_efield(g, rc, ph, u, i, j, k, e0, e1, e2);
            a += (e0 * e0 + e1 * e1 + e2 * e2) * ens_node_volume(g, i, j, k);
        }
        part[v] = a;
    }
    const double t = ens_tree_sum(part);
    if (threadIdx.x == 0) out[bid * ncol + nsp] = 0.5 * ENS_EPS_0 * t;
}

}  // namespace espic

/* ======================================================================== */
/* C-ABI                                                                    */
using namespace espic;

struct espic_ensemble {
    int nbox = 0, nsp = 0, device = 0, sm_count = 0;
    cudaStream_t stream = nullptr;
    double dt = 0;
    uint64_t seed = 0x5eed;
    std::vector<EnsBox> boxes;
    std::vector<int32_t> box_id; /* the id that keys each box's random streams (default: its index) */
    std::vector<EnsSeg> segs; /* [box][species] */
    std::vector<double> mass, charge, mpw0;
    int64_t total_nodes = 0, total_cap = 0;
    EnsBox *d_boxes = nullptr;
    EnsSeg *d_segs = nullptr;
    double *d_mass = nullptr, *d_mpw = nullptr;
    double *phi = nullptr, *rho = nullptr;
    float4 *ef4 = nullptr;
    float *ecor = nullptr, *res = nullptr;
    unsigned long long *acc = nullptr;
    int32_t *cell = nullptr;
    float *off = nullptr, *vel = nullptr;
    int4 *d_work = nullptr;
    int nwork = 0;
    bool work_valid = false;
    int *d_order = nullptr, *d_counter = nullptr, *d_err = nullptr;
    EnsStat *d_stat = nullptr;
    double *d_scratch = nullptr;
    size_t scratch_bytes = 0;
    int max_it = 10000;
    double tol = 1e-4, omega_req = 0;
    int chunk = 4096, push_threads = 256, solve_threads = 1024, cluster = 8;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int64_t nlaunch = 0, steps = 0;
};

static int efail(int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    return espic_internal_fail(code, buf);
}

#define ECK(call)                                                                                       \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return efail(ESPIC_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

#define ENSEMBLE(h)                                                        \
    if (!(h)) return efail(ESPIC_ERR_ARG, "null ensemble handle");         \
    espic_ensemble &E = *(h);                                              \
    if (cudaSetDevice(E.device) != cudaSuccess) return efail(ESPIC_ERR_CUDA, "cudaSetDevice failed")

template <typename T>
static cudaError_t ens_alloc(T **p, size_t count) {
    cudaError_t e = cudaMalloc((void **)p, count * sizeof(T) + 16);
    if (e == cudaSuccess) e = cudaMemset(*p, 0, count * sizeof(T) + 16);
    return e;
}

static void ens_free(espic_ensemble *e) {
    if (e->exec) cudaGraphExecDestroy(e->exec);
    if (e->graph) cudaGraphDestroy(e->graph);
    void *ptrs[] = {e->d_boxes, e->d_segs, e->d_mass, e->d_mpw, e->phi, e->rho, e->ef4, e->ecor, e->res, e->acc,
                    e->cell, e->off, e->vel, e->d_work, e->d_order, e->d_counter, e->d_err, e->d_stat,
                    e->d_scratch};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

/* optimal red-black SOR factor of the Dirichlet 7-point Laplacian on a box
 * (Young): rho_J = sum c_d cos(pi / (n_d - 1)) / sum c_d */
static double omega_opt(const Geo &g) {
    double c[3], num = 0, den = 0;
    int n[3] = {g.ni, g.nj, g.nk};
    for (int d = 0; d < 3; d++) {
        c[d] = 1.0 / (g.dh[d] * g.dh[d]);
        num += c[d] * cos(3.14159265358979323846 / (n[d] - 1));
        den += c[d];
    }
    double rj = num / den;
    return 2.0 / (1.0 + sqrt(1.0 - rj * rj));
}

static void ens_set_omega(espic_ensemble &E) {
    for (EnsBox &b : E.boxes) b.omega = E.omega_req > 0 ? E.omega_req : omega_opt(b.g);
}

static int ens_upload_tables(espic_ensemble &E) {
    ECK(cudaMemcpyAsync(E.d_boxes, E.boxes.data(), E.boxes.size() * sizeof(EnsBox), cudaMemcpyHostToDevice,
                        E.stream));
    ECK(cudaMemcpyAsync(E.d_segs, E.segs.data(), E.segs.size() * sizeof(EnsSeg), cudaMemcpyHostToDevice,
                        E.stream));
    ECK(cudaStreamSynchronize(E.stream));
    return ESPIC_OK;
}

static void ens_drop_graph(espic_ensemble &E) {
    if (E.exec) cudaGraphExecDestroy(E.exec);
    if (E.graph) cudaGraphDestroy(E.graph);
    E.exec = nullptr;
    E.graph = nullptr;
}

/* the flattened work list: chunks of at most E.chunk particles, each inside
 * one segment, the largest segments first */
static int ens_build_work(espic_ensemble &E) {
    std::vector<int> sidx(E.segs.size());
    for (size_t i = 0; i < sidx.size(); i++) sidx[i] = (int)i;
    std::stable_sort(sidx.begin(), sidx.end(), [&](int a, int b) { return E.segs[a].n > E.segs[b].n; });
    std::vector<int4> work;
    for (int si : sidx) {
        const EnsSeg &s = E.segs[si];
        for (int64_t st = 0; st < s.n; st += E.chunk) {
            int64_t c = s.n - st < E.chunk ? s.n - st : E.chunk;
            work.push_back(make_int4(si, (int)st, (int)c, 0));
        }
    }
    if (E.d_work) cudaFree(E.d_work);
    E.d_work = nullptr;
    E.nwork = (int)work.size();
    if (E.nwork) {
        ECK(cudaMalloc(&E.d_work, work.size() * sizeof(int4)));
        ECK(cudaMemcpy(E.d_work, work.data(), work.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    E.work_valid = true;
    return ESPIC_OK;
}

static int ens_push_blocks(espic_ensemble &E) {
    int64_t b = (int64_t)E.sm_count * (2048 / E.push_threads);
    return (int)(E.nwork < b ? (E.nwork > 0 ? E.nwork : 1) : b);
}

/* the solve launch: clusters of E.cluster CTAs, as many as can be resident
 * (one box each at a time), at most one per box */
static cudaError_t ens_launch_solve(espic_ensemble &E, int solve) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = E.cluster;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(E.solve_threads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = E.stream;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cfg.gridDim = dim3(E.cluster);
    int ncl = 0;
    cudaError_t ce = cudaOccupancyMaxActiveClusters(&ncl, (void *)k_ens_solve, &cfg);
    if (ce != cudaSuccess || ncl < 1) ncl = E.sm_count / E.cluster > 0 ? E.sm_count / E.cluster : 1;
    if (ncl > E.nbox) ncl = E.nbox;
    cfg.gridDim = dim3(ncl * E.cluster);
    return cudaLaunchKernelEx(&cfg, k_ens_solve, (const EnsBox *)E.d_boxes, (const EnsSeg *)E.d_segs, E.nsp,
                              (const int *)E.d_order, E.nbox, E.d_counter, E.phi, E.rho, E.ecor, E.res, E.ef4, E.acc,
                              E.total_nodes, E.max_it, E.tol, solve, E.d_stat, E.d_err);
}

/* enqueue one phase sequence: [push +] deposit, then rho / solve / E */
static int ens_enqueue(espic_ensemble &E, bool push, bool solve) {
    if (!E.work_valid) {
        int rc = ens_build_work(E);
        if (rc) return rc;
    }
    launch_ens_push(E.stream, push, ens_push_blocks(E), E.push_threads, E.d_boxes, E.d_segs, E.d_work, E.nwork,
                    E.ef4, E.cell, E.off, E.vel, E.total_cap, E.acc, E.total_nodes, E.d_err);
    ECK(cudaMemsetAsync(E.d_counter, 0, sizeof(int), E.stream));
    ECK(ens_launch_solve(E, solve ? 1 : 0));
    E.nlaunch += E.nwork ? 2 : 1;
    cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return efail(ESPIC_ERR_CUDA, "ensemble launch: %s", cudaGetErrorString(le));
    return ESPIC_OK;
}

static int ens_take_errors(espic_ensemble &E) {
    int bits = 0;
    ECK(cudaMemcpyAsync(&bits, E.d_err, sizeof(int), cudaMemcpyDeviceToHost, E.stream));
    ECK(cudaStreamSynchronize(E.stream));
    if (bits) ECK(cudaMemsetAsync(E.d_err, 0, sizeof(int), E.stream));
    if (bits & DERR_NONFINITE) return efail(ESPIC_ERR_NONFINITE, "non-finite value in the ensemble step");
    return ESPIC_OK;
}

extern "C" int espic_ensemble_create(int nbox, const int32_t *nodes, const double *x0, const double *xm,
                                     int nspecies, const double *mass, const double *charge, const double *mpw0,
                                     const int64_t *capacity, double dt, espic_ensemble **out) {
    if (!out || !nodes || !x0 || !xm || !mass || !charge || !mpw0 || !capacity)
        return efail(ESPIC_ERR_ARG, "null argument");
    *out = nullptr;
    if (nbox < 1 || nspecies < 1 || nspecies > 8) return efail(ESPIC_ERR_ARG, "need nbox >= 1 and 1..8 species");
    if (!(dt > 0)) return efail(ESPIC_ERR_ARG, "dt must be positive");
    espic_ensemble *e = new espic_ensemble();
    espic_ensemble &E = *e;
    E.nbox = nbox;
    E.nsp = nspecies;
    E.dt = dt;
    cudaGetDevice(&E.device);
    cudaDeviceGetAttribute(&E.sm_count, cudaDevAttrMultiProcessorCount, E.device);
    E.mass.assign(mass, mass + nspecies);
    E.charge.assign(charge, charge + nspecies);
    E.mpw0.assign(mpw0, mpw0 + (size_t)nbox * nspecies);
    int64_t node0 = 0, p0 = 0;
    for (int b = 0; b < nbox; b++) {
        EnsBox bx{};
        int n3[3] = {nodes[3 * b], nodes[3 * b + 1], nodes[3 * b + 2]};
        for (int d = 0; d < 3; d++) {
            if (n3[d] < 3 || n3[d] > 1024) {
                ens_free(e);
                return efail(ESPIC_ERR_ARG, "box %d: node counts must be in [3, 1024]", b);
            }
            if (!(xm[3 * b + d] > x0[3 * b + d])) {
                ens_free(e);
                return efail(ESPIC_ERR_ARG, "box %d: xm must exceed x0", b);
            }
        }
        bx.g.ni = n3[0];
        bx.g.nj = n3[1];
        bx.g.nk = n3[2];
        for (int d = 0; d < 3; d++) {
            bx.g.x0[d] = x0[3 * b + d];
            bx.g.xm[d] = xm[3 * b + d];
            bx.g.dh[d] = (xm[3 * b + d] - x0[3 * b + d]) / (n3[d] - 1);
            bx.dtdh[d] = (float)(dt / bx.g.dh[d]);
        }
        bx.nn = (int64_t)n3[0] * n3[1] * n3[2];
        bx.node0 = node0;
        node0 += (bx.nn + 63) / 64 * 64;
        E.boxes.push_back(bx);
        for (int s = 0; s < nspecies; s++) {
            int64_t cap = capacity[(size_t)b * nspecies + s];
            if (cap < 0 || cap > 0x7fffffffLL) {
                ens_free(e);
                return efail(ESPIC_ERR_ARG, "capacity must be in [0, 2^31)");
            }
            EnsSeg sg{};
            sg.box = b;
            sg.sp = s;
            sg.p0 = p0;
            sg.n = 0;
            sg.cap = cap;
            sg.unit = mpw0[(size_t)b * nspecies + s] / 8388608.0;
            sg.q = charge[s];
            sg.qmdt = (float)(charge[s] / mass[s] * dt);
            p0 += (cap + 63) / 64 * 64;
            E.segs.push_back(sg);
        }
    }
    E.total_nodes = node0;
    E.total_cap = p0 > 0 ? p0 : 64;
    ens_set_omega(E);
    cudaError_t ce = cudaStreamCreateWithFlags(&E.stream, cudaStreamNonBlocking);
    const int64_t TN = E.total_nodes, TC = E.total_cap;
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_boxes, (size_t)nbox);
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_segs, E.segs.size());
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_mass, (size_t)nspecies);
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_mpw, E.mpw0.size());
    if (ce == cudaSuccess) ce = ens_alloc(&E.phi, (size_t)TN);
    if (ce == cudaSuccess) ce = ens_alloc(&E.rho, (size_t)TN);
    if (ce == cudaSuccess) ce = ens_alloc(&E.ef4, (size_t)TN);
    if (ce == cudaSuccess) ce = ens_alloc(&E.ecor, (size_t)TN);
    if (ce == cudaSuccess) ce = ens_alloc(&E.res, (size_t)TN);
    if (ce == cudaSuccess) ce = ens_alloc(&E.acc, (size_t)TN * nspecies);
    if (ce == cudaSuccess) ce = ens_alloc(&E.cell, (size_t)TC);
    if (ce == cudaSuccess) ce = ens_alloc(&E.off, (size_t)TC * 3);
    if (ce == cudaSuccess) ce = ens_alloc(&E.vel, (size_t)TC * 3);
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_order, (size_t)nbox);
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_counter, 1);
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_err, 1);
    if (ce == cudaSuccess) ce = ens_alloc(&E.d_stat, (size_t)nbox);
    if (ce != cudaSuccess) {
        ens_free(e);
        return efail(ESPIC_ERR_CUDA, "ensemble allocation: %s", cudaGetErrorString(ce));
    }
    /* boxes in decreasing node count: the solve claims big boxes first */
    std::vector<int> order(nbox);
    for (int b = 0; b < nbox; b++) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return E.boxes[a].nn > E.boxes[b].nn; });
    cudaMemcpy(E.d_order, order.data(), nbox * sizeof(int), cudaMemcpyHostToDevice);
    cudaMemcpy(E.d_mass, E.mass.data(), nspecies * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(E.d_mpw, E.mpw0.data(), E.mpw0.size() * sizeof(double), cudaMemcpyHostToDevice);
    int rc = ens_upload_tables(E);
    if (rc) {
        ens_free(e);
        return rc;
    }
    *out = e;
    return ESPIC_OK;
}

extern "C" void espic_ensemble_destroy(espic_ensemble *e) {
    if (!e) return;
    cudaSetDevice(e->device);
    cudaStreamSynchronize(e->stream);
    ens_free(e);
}

#define SEG(box, sp)                                                                              \
    if ((box) < 0 || (box) >= E.nbox || (sp) < 0 || (sp) >= E.nsp)                               \
        return efail(ESPIC_ERR_ARG, "box %d / species %d out of range", (int)(box), (int)(sp));  \
    EnsSeg &S = E.segs[(size_t)(box)*E.nsp + (sp)];                                               \
    const EnsBox &BX = E.boxes[(box)]

extern "C" int espic_ensemble_set_particles(espic_ensemble *h, int box, int sp, const double *P, int64_t stride,
                                            int64_t n) {
    ENSEMBLE(h);
    SEG(box, sp);
    if (n < 0 || (n > 0 && (!P || stride < n))) return efail(ESPIC_ERR_ARG, "bad particle block");
    if (n > S.cap) return efail(ESPIC_ERR_CAPACITY, "%lld particles exceed the capacity", (long long)n);
    if (n > 0) {
        size_t bytes = (size_t)7 * n * sizeof(double);
        if (E.scratch_bytes < bytes) {
            if (E.d_scratch) cudaFree(E.d_scratch);
            E.d_scratch = nullptr;
            E.scratch_bytes = 0;
            ECK(cudaMalloc(&E.d_scratch, bytes));
            E.scratch_bytes = bytes;
        }
        ECK(cudaMemcpy2DAsync(E.d_scratch, n * sizeof(double), P, stride * sizeof(double), n * sizeof(double), 7,
                              cudaMemcpyHostToDevice, E.stream));
        launch_to_mixed_raw(E.stream, BX.g, E.d_scratch, n, n, S.p0, E.cell, E.off, E.vel, E.total_cap);
        E.nlaunch++;
        ECK(cudaGetLastError());
        ECK(cudaStreamSynchronize(E.stream));
    }
    S.n = n;
    E.work_valid = false;
    ens_drop_graph(E);
    return ens_upload_tables(E);
}

extern "C" int espic_ensemble_load_box(espic_ensemble *h, int box, int sp, const double x1[3], const double x2[3],
                                       int64_t num_mp) {
    ENSEMBLE(h);
    SEG(box, sp);
    if (!x1 || !x2) return efail(ESPIC_ERR_ARG, "null argument");
    if (num_mp < 0 || num_mp > S.cap) return efail(ESPIC_ERR_CAPACITY, "num_mp exceeds the capacity");
    for (int d = 0; d < 3; d++)
        if (x1[d] < BX.g.x0[d] || x2[d] > BX.g.xm[d] || !(x2[d] > x1[d]))
            return efail(ESPIC_ERR_ARG, "load region must lie inside the box");
    const uint64_t id = E.box_id.empty() ? (uint64_t)box : (uint64_t)E.box_id[box];
    uint64_t stream = ((uint64_t)(0x40000 + id * E.nsp + sp)) << 32;
    if (num_mp > 0) {
        k_ens_load<<<blocks_for(num_mp, 256), 256, 0, E.stream>>>(BX.g, make_double3(x1[0], x1[1], x1[2]),
                                                                  make_double3(x2[0], x2[1], x2[2]), num_mp, E.seed,
                                                                  stream, S.p0, E.cell, E.off, E.vel, E.total_cap);
        E.nlaunch++;
        ECK(cudaGetLastError());
    }
    S.n = num_mp;
    E.work_valid = false;
    ens_drop_graph(E);
    return ens_upload_tables(E);
}

extern "C" int espic_ensemble_set_box_ids(espic_ensemble *h, const int32_t *ids) {
    ENSEMBLE(h);
    if (!ids) {
        E.box_id.clear();
        return ESPIC_OK;
    }
    for (int b = 0; b < E.nbox; b++)
        if (ids[b] < 0 || ids[b] >= (1 << 24)) return efail(ESPIC_ERR_ARG, "box id %d out of range", ids[b]);
    E.box_id.assign(ids, ids + E.nbox);
    return ESPIC_OK;
}

extern "C" int espic_partition_boxes(int nbox, const double *work, int nparts, int32_t *owner, double *load) {
    if (nbox < 0 || nparts < 1 || (nbox > 0 && (!work || !owner)))
        return efail(ESPIC_ERR_ARG, "bad partition arguments");
    for (int b = 0; b < nbox; b++)
        if (!(work[b] >= 0)) return efail(ESPIC_ERR_ARG, "box %d: work must be finite and >= 0", b);
    /* largest work first (ties by box index), each to the least loaded part
     * (ties to the lowest part): deterministic on every rank */
    std::vector<int> order(nbox);
    for (int b = 0; b < nbox; b++) order[b] = b;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return work[a] > work[b]; });
    std::vector<double> L(nparts, 0.0);
    for (int b : order) {
        int best = 0;
        for (int r = 1; r < nparts; r++)
            if (L[r] < L[best]) best = r;
        owner[b] = best;
        L[best] += work[b];
    }
    if (load)
        for (int r = 0; r < nparts; r++) load[r] = L[r];
    return ESPIC_OK;
}

extern "C" int espic_ensemble_set_seed(espic_ensemble *h, uint64_t seed) {
    ENSEMBLE(h);
    E.seed = seed;
    return ESPIC_OK;
}

extern "C" int espic_ensemble_get_particles(espic_ensemble *h, int box, int sp, double *P, int64_t stride,
                                            int64_t cap, int64_t *n_out) {
    ENSEMBLE(h);
    SEG(box, sp);
    if (n_out) *n_out = S.n;
    if (S.n == 0 || !P) return ESPIC_OK; /* P = NULL: count only */
    if (cap < S.n || stride < S.n) return efail(ESPIC_ERR_ARG, "buffer smaller than the particle count");
    size_t bytes = (size_t)7 * S.n * sizeof(double);
    if (E.scratch_bytes < bytes) {
        if (E.d_scratch) cudaFree(E.d_scratch);
        E.d_scratch = nullptr;
        E.scratch_bytes = 0;
        ECK(cudaMalloc(&E.d_scratch, bytes));
        E.scratch_bytes = bytes;
    }
    launch_from_mixed_raw(E.stream, BX.g, E.cell, E.off, E.vel, E.total_cap, S.p0, S.n, E.mpw0[(size_t)box * E.nsp + sp],
                          E.d_scratch, S.n);
    E.nlaunch++;
    ECK(cudaGetLastError());
    ECK(cudaMemcpy2DAsync(P, stride * sizeof(double), E.d_scratch, S.n * sizeof(double), S.n * sizeof(double), 7,
                          cudaMemcpyDeviceToHost, E.stream));
    ECK(cudaStreamSynchronize(E.stream));
    return ESPIC_OK;
}

extern "C" int espic_ensemble_set_solver(espic_ensemble *h, int max_it, double tol, double omega) {
    ENSEMBLE(h);
    if (max_it < 0 || !(tol > 0) || omega < 0 || omega >= 2) return efail(ESPIC_ERR_ARG, "bad solver controls");
    E.max_it = max_it;
    E.tol = tol;
    E.omega_req = omega;
    ens_set_omega(E);
    ens_drop_graph(E);
    return ens_upload_tables(E);
}

extern "C" int espic_ensemble_set_launch(espic_ensemble *h, int chunk, int push_threads, int solve_threads,
                                         int cluster) {
    ENSEMBLE(h);
    bool okp = push_threads == 128 || push_threads == 256 || push_threads == 512;
    bool oks = solve_threads == 256 || solve_threads == 512 || solve_threads == 1024;
    bool okc = cluster == 1 || cluster == 2 || cluster == 4 || cluster == 8;
    if (chunk < 256 || chunk > (1 << 24) || !okp || !oks || !okc) return efail(ESPIC_ERR_ARG, "bad launch shape");
    if (chunk != E.chunk) E.work_valid = false;
    E.chunk = chunk;
    E.push_threads = push_threads;
    E.solve_threads = solve_threads;
    E.cluster = cluster;
    ens_drop_graph(E);
    return ESPIC_OK;
}

extern "C" int espic_ensemble_get_launch(espic_ensemble *h, int *chunk, int *push_threads, int *solve_threads,
                                         int *cluster) {
    ENSEMBLE(h);
    if (chunk) *chunk = E.chunk;
    if (push_threads) *push_threads = E.push_threads;
    if (solve_threads) *solve_threads = E.solve_threads;
    if (cluster) *cluster = E.cluster;
    return ESPIC_OK;
}

/* the state before the first step of ch2/Main.cpp: deposit, charge density,
 * solve, E */
extern "C" int espic_ensemble_prepare(espic_ensemble *h) {
    ENSEMBLE(h);
    int rc = ens_enqueue(E, false, true);
    if (rc) return rc;
    return ens_take_errors(E);
}

/* nsteps steps (push + deposit, charge, solve, E), each one launch of the
 * step's CUDA graph; asynchronous unless an error must be reported */
extern "C" int espic_ensemble_step(espic_ensemble *h, int nsteps) {
    ENSEMBLE(h);
    if (nsteps < 0) return efail(ESPIC_ERR_ARG, "nsteps must be >= 0");
    if (!E.work_valid) {
        int rc = ens_build_work(E);
        if (rc) return rc;
    }
    if (!E.exec) {
        ECK(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal));
        int64_t before = E.nlaunch;
        int rc = ens_enqueue(E, true, true);
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(E.stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (ce != cudaSuccess) return efail(ESPIC_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ce));
        E.nlaunch = before;
        E.graph = g;
        ECK(cudaGraphInstantiate(&E.exec, g, 0));
    }
    for (int s = 0; s < nsteps; s++) {
        ECK(cudaGraphLaunch(E.exec, E.stream));
        E.nlaunch += E.nwork ? 2 : 1;
        E.steps++;
    }
    return ESPIC_OK;
}

/* the same step as direct launches (no graph) */
extern "C" int espic_ensemble_step_direct(espic_ensemble *h, int nsteps) {
    ENSEMBLE(h);
    for (int s = 0; s < nsteps; s++) {
        int rc = ens_enqueue(E, true, true);
        if (rc) return rc;
        E.steps++;
    }
    return ESPIC_OK;
}

extern "C" int espic_ensemble_sync(espic_ensemble *h) {
    ENSEMBLE(h);
    return ens_take_errors(E);
}

extern "C" void *espic_ensemble_stream(espic_ensemble *h) { return h ? (void *)h->stream : nullptr; }

extern "C" int espic_ensemble_launches(espic_ensemble *h, int64_t *n) {
    ENSEMBLE(h);
    if (n) *n = E.nlaunch;
    return ESPIC_OK;
}

extern "C" int espic_ensemble_status(espic_ensemble *h, int32_t *sweeps, int32_t *converged, double *residual) {
    ENSEMBLE(h);
    std::vector<EnsStat> st(E.nbox);
    ECK(cudaMemcpyAsync(st.data(), E.d_stat, E.nbox * sizeof(EnsStat), cudaMemcpyDeviceToHost, E.stream));
    ECK(cudaStreamSynchronize(E.stream));
    for (int b = 0; b < E.nbox; b++) {
        if (sweeps) sweeps[b] = st[b].sweeps;
        if (converged) converged[b] = st[b].converged;
        if (residual) residual[b] = st[b].residual;
    }
    return ens_take_errors(E);
}

/* field of one box: ESPIC_FIELD_PHI, RHO, EF ([nn][3]) or DEN of species sp
 * (deposited from the current particles) */
extern "C" int espic_ensemble_read(espic_ensemble *h, int box, int field, int sp, double *out) {
    ENSEMBLE(h);
    if (box < 0 || box >= E.nbox || !out) return efail(ESPIC_ERR_ARG, "bad box or null output");
    const EnsBox &B = E.boxes[box];
    size_t nn = (size_t)B.nn;
    if (field == ESPIC_FIELD_PHI || field == ESPIC_FIELD_RHO) {
        const double *src = (field == ESPIC_FIELD_PHI ? E.phi : E.rho) + B.node0;
        ECK(cudaMemcpyAsync(out, src, nn * sizeof(double), cudaMemcpyDeviceToHost, E.stream));
        ECK(cudaStreamSynchronize(E.stream));
        return ESPIC_OK;
    }
    size_t need = (field == ESPIC_FIELD_EF ? 3 : 1) * nn * sizeof(double);
    if (E.scratch_bytes < need) {
        if (E.d_scratch) cudaFree(E.d_scratch);
        E.d_scratch = nullptr;
        E.scratch_bytes = 0;
        ECK(cudaMalloc(&E.d_scratch, need));
        E.scratch_bytes = need;
    }
    if (field == ESPIC_FIELD_EF) {
        k_ens_efield64<<<blocks_for((int64_t)nn, 256), 256, 0, E.stream>>>(B.g, E.phi + B.node0, E.d_scratch);
        E.nlaunch++;
    } else if (field == ESPIC_FIELD_DEN) {
        if (sp < 0 || sp >= E.nsp) return efail(ESPIC_ERR_ARG, "species out of range");
        /* deposit every box into the (clear) accumulators, convert this one,
         * clear them again */
        if (!E.work_valid) {
            int rc = ens_build_work(E);
            if (rc) return rc;
        }
        launch_ens_push(E.stream, false, ens_push_blocks(E), E.push_threads, E.d_boxes, E.d_segs, E.d_work,
                        E.nwork, E.ef4, E.cell, E.off, E.vel, E.total_cap, E.acc, E.total_nodes, E.d_err);
        const EnsSeg &S = E.segs[(size_t)box * E.nsp + sp];
        k_ens_density<<<blocks_for((int64_t)nn, 256), 256, 0, E.stream>>>(
            B.g, E.acc + (int64_t)sp * E.total_nodes + B.node0, S.unit, E.d_scratch);
        E.nlaunch += 2;
        ECK(cudaGetLastError());
        ECK(cudaMemsetAsync(E.acc, 0, (size_t)E.total_nodes * E.nsp * sizeof(unsigned long long), E.stream));
    } else {
        return efail(ESPIC_ERR_ARG, "field %d cannot be read from an ensemble", field);
    }
    ECK(cudaGetLastError());
    ECK(cudaMemcpyAsync(out, E.d_scratch, need, cudaMemcpyDeviceToHost, E.stream));
    ECK(cudaStreamSynchronize(E.stream));
    return ESPIC_OK;
}

/* out[box][0..nsp) kinetic energy per species, out[box][nsp] field energy */
extern "C" int espic_ensemble_diag(espic_ensemble *h, double *out) {
    ENSEMBLE(h);
    if (!out) return efail(ESPIC_ERR_ARG, "null output");
    size_t need = (size_t)E.nbox * (E.nsp + 1) * sizeof(double);
    if (E.scratch_bytes < need) {
        if (E.d_scratch) cudaFree(E.d_scratch);
        E.d_scratch = nullptr;
        E.scratch_bytes = 0;
        ECK(cudaMalloc(&E.d_scratch, need));
        E.scratch_bytes = need;
    }
    k_ens_diag<<<E.nbox, 256, 0, E.stream>>>(E.d_boxes, E.d_segs, E.nsp, E.d_mass, E.d_mpw, E.phi, E.vel,
                                            E.total_cap, E.d_scratch);
    E.nlaunch++;
    ECK(cudaGetLastError());
    ECK(cudaMemcpyAsync(out, E.d_scratch, need, cudaMemcpyDeviceToHost, E.stream));
    ECK(cudaStreamSynchronize(E.stream));
    return ens_take_errors(E);
}

/* Autotuner: times every candidate launch shape on real steps (results do not
 * depend on the shape: per-particle pushes, integer deposits, colour-ordered
 * sweeps, fixed-width reductions) with CUDA events around the two phases, and
 * keeps the fastest chunk / push block for the push phase and the fastest
 * cluster size / solve block for the solve phase.  Consumes 27 steps. */
extern "C" int espic_ensemble_autotune(espic_ensemble *h, int *chunk, int *push_threads, int *solve_threads,
                                       double *push_ms, double *solve_ms) {
    ENSEMBLE(h);
    const int chunks[] = {1024, 2048, 4096, 8192, 16384};
    const int pts[] = {128, 256, 512};
    const int sts[] = {256, 512, 1024};
    const int cls[] = {1, 2, 4, 8};
    cudaEvent_t a, b, c;
    ECK(cudaEventCreate(&a));
    ECK(cudaEventCreate(&b));
    ECK(cudaEventCreate(&c));
    float best_push = 1e30f, best_solve = 1e30f;
    int bc = E.chunk, bp = E.push_threads, bs = E.solve_threads;
    for (int ci = 0; ci < 5; ci++)
        for (int pi = 0; pi < 3; pi++) {
            E.chunk = chunks[ci];
            E.push_threads = pts[pi];
            E.work_valid = false;
            int rc = ens_build_work(E);
            if (rc) return rc;
            ECK(cudaEventRecord(a, E.stream));
            launch_ens_push(E.stream, true, ens_push_blocks(E), E.push_threads, E.d_boxes, E.d_segs, E.d_work,
                            E.nwork, E.ef4, E.cell, E.off, E.vel, E.total_cap, E.acc, E.total_nodes, E.d_err);
            ECK(cudaEventRecord(b, E.stream));
            ECK(cudaMemsetAsync(E.d_counter, 0, sizeof(int), E.stream));
            ECK(ens_launch_solve(E, 1));
            E.nlaunch += 2;
            E.steps++;
            ECK(cudaGetLastError());
            ECK(cudaEventSynchronize(b));
            float ms = 0;
            ECK(cudaEventElapsedTime(&ms, a, b));
            if (ms < best_push) {
                best_push = ms;
                bc = E.chunk;
                bp = E.push_threads;
            }
        }
    E.chunk = bc;
    E.push_threads = bp;
    E.work_valid = false;
    int rc = ens_build_work(E);
    if (rc) return rc;
    int bcl = E.cluster;
    for (int ki = 0; ki < 4; ki++)
        for (int si = 0; si < 3; si++) {
            E.cluster = cls[ki];
            E.solve_threads = sts[si];
            launch_ens_push(E.stream, true, ens_push_blocks(E), E.push_threads, E.d_boxes, E.d_segs, E.d_work,
                            E.nwork, E.ef4, E.cell, E.off, E.vel, E.total_cap, E.acc, E.total_nodes, E.d_err);
            ECK(cudaMemsetAsync(E.d_counter, 0, sizeof(int), E.stream));
            ECK(cudaEventRecord(b, E.stream));
            ECK(ens_launch_solve(E, 1));
            ECK(cudaEventRecord(c, E.stream));
            E.nlaunch += 2;
            E.steps++;
            ECK(cudaGetLastError());
            ECK(cudaEventSynchronize(c));
            float ms = 0;
            ECK(cudaEventElapsedTime(&ms, b, c));
            if (ms < best_solve) {
                best_solve = ms;
                bs = E.solve_threads;
                bcl = E.cluster;
            }
        }
    E.solve_threads = bs;
    E.cluster = bcl;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaEventDestroy(c);
    ens_drop_graph(E);
    if (chunk) *chunk = E.chunk;
    if (push_threads) *push_threads = E.push_threads;
    if (solve_threads) *solve_threads = E.solve_threads;
    if (push_ms) *push_ms = best_push;
    if (solve_ms) *solve_ms = best_solve;
    return ens_take_errors(E);
}

extern "C" int espic_ensemble_steps_taken(espic_ensemble *h, int64_t *steps) {
    ENSEMBLE(h);
    if (steps) *steps = E.steps;
    return ESPIC_OK;
}
