/*
 * espic_internal.h -- device data layout and kernel launchers shared by the
 * translation units of libespic.  Not part of the public interface
 * (include/espic.h is).
 *
 * Data layout in HBM (one World):
 *  - node fields: linear arrays in U order, u = k*ni*nj + j*ni + i
 *    (ch3/ver2/Field.h:161): phi, rho, node_vol (f64); ef interleaved [nn][3]
 *    f64 plus an f32 copy ef4 [nn] float4 (x, y, z, 0) for the mixed push;
 *    object_id and Neumann chain targets (int32).
 *  - particles, FP64 plain form: one block P[7][cap] f64 = x, y, z, vx, vy,
 *    vz, mpw (row stride = cap).
 *  - particles, mixed form: cell key int32 (i | j<<10 | k<<20), in-cell
 *    offsets f32 [3][cap] in [0,1), velocity f32 [3][cap] (m/s): 28 B each;
 *    the macroparticle weight is the species' mpw0.
 *  - per species: int64 fixed-point deposit accumulator [nn], den and den_ave
 *    f64 [nn], a dead-particle bit mask [cap/32] and per-tile dead counts.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace espic {

/* error bits accumulated on the device, read at synchronising calls */
enum : int {
    DERR_CAPACITY = 1,   /* particle buffer full: injection or load truncated */
    DERR_NONFINITE = 2,  /* NaN / Inf met in a solve */
    DERR_FIXED_RANGE = 4, /* a weight too large for the fixed-point scale */
    DERR_TIMEOUT = 8,     /* a bounded wait on an asynchronous copy ran out */
    DERR_SORT = 16,       /* a sort slot named no particle of the species */
    DERR_DSMC = 32,       /* a collision partner outside the domain, or replayed uniforms ran out */
    DERR_NEUTRAL = 64     /* moments / MCC: a particle outside the grid, a non-finite moment, or replayed
                             uniforms out of range */
};

struct Geo {
    int ni, nj, nk;
    double x0[3], xm[3], dh[3];
};

/* particles per dead-count tile of the compaction */
constexpr int TILE_PARTICLES = 32768;

/* cells per edge of a tile of the mixed form's sort order */
constexpr int TILE_CELLS = 8;
__host__ __device__ inline int tile_count(int ncell) { return (ncell + TILE_CELLS - 1) / TILE_CELLS; }

/* sampled velocity moments of a ch4 species: n, n u, n v, n w, n u u, n v v, n w w */
constexpr int NMOM = 7;

struct SolveStatus {
    int converged;
    int iterations;
    int inner_iterations;
    int fallback_sweeps; /* Gauss-Seidel sweeps after a failed inner PCG (Newton-PCG) */
    double residual;
    long long solves;       /* running totals, added by every solve */
    long long outer_total;
    long long inner_total;
};

/* ---------------- counter-based RNG: Philox4x32-10 (Salmon et al. 2011) */
__host__ __device__ inline void philox4x32(uint32_t c[4], uint32_t k0, uint32_t k1) {
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

__host__ __device__ inline double u53(uint32_t a, uint32_t b) {
    uint64_t x = (((uint64_t)a << 32) | b) >> 11;
    return (double)x * (1.0 / 9007199254740992.0);
}

/* uniform number `index` of stream `stream` under key `seed`, in [0,1) */
__host__ __device__ inline double philox_uniform(uint64_t seed, uint64_t stream, uint64_t index) {
    uint64_t blk = index >> 1;
    uint32_t c[4] = {(uint32_t)blk, (uint32_t)(blk >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
    philox4x32(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    return (index & 1) ? u53(c[2], c[3]) : u53(c[0], c[1]);
}

/* ---------------- batched ensemble of independent boxes ---------------- */
/* One box: its geometry and where its nodes sit in the concatenated node
 * fields of the ensemble. */
struct EnsBox {
    Geo g;
    int64_t node0; /* first node of the box in the concatenated node fields */
    int64_t nn;
    double omega;  /* red-black SOR relaxation factor */
    float dtdh[3]; /* dt / dh per axis */
    int pad;
};

/* The particles of one species in one box: rows [p0, p0 + n) of the
 * concatenated mixed-form particle rows. */
struct EnsSeg {
    int box, sp;
    int64_t p0, n, cap;
    double unit; /* real particles per deposit count: mpw0 * 2^-23 */
    double q;    /* charge */
    float qmdt;  /* q / m dt */
    int pad;
};

struct EnsStat {
    int sweeps, converged;
    double residual;
};

/* ---------------- launchers (stream-ordered, asynchronous) ------------- */
struct Species;
struct World;

/* k_fp64.cu */
void launch_objects_sphere(World &w, const double c[3], double radius, double phi_s);
void launch_objects_inlet(World &w);
void launch_targets(World &w);
/* computeEF.  full = false lets a world whose species are all in the mixed
 * form write ef4 and the inlet planes of ef only; ensure_ef64 completes ef
 * before a float64 consumer reads it */
void launch_efield(World &w, bool full = true);
void ensure_ef64(World &w);
void launch_push_fp64(World &w, Species &s, bool deposit);
void launch_deposit_fp64(World &w, Species &s);
void launch_compact(World &w, Species &s);
void launch_density(World &w, Species &s);
void launch_int_excl_scan(cudaStream_t st, int32_t *x, int64_t n, int32_t *bsum);
int64_t int_scan_blocks(int64_t n);
void launch_dsmc(World &w, Species &s, double dt, const double *d_u, int64_t nu, const int64_t *d_cell_off);
/* ch4 species moments and MCC charge exchange (float64 form) */
void launch_moments(World &w, Species &s);
void launch_gas_props(World &w, Species &s);
void launch_mpc(World &w, Species &s);
void launch_mcc(World &w, Species &src, const Species &tgt, double dt, const double *d_u, int64_t nu,
                const int64_t *d_off, unsigned long long *d_ncol);
/* ch4 Species::advance of a neutral species (sphere diffuse reflection) */
void launch_advance_ch4(World &w, Species &s, double dt, const double *d_pdt, const double *d_u, int64_t nu,
                        const int64_t *d_off);
/* ch4 Species::advance of a charged species: struck ions create particles
 * in neu and sph (which may be one species) */
void launch_advance_ch4_ions(World &w, Species &s, Species &neu, Species &sph, double dt, const double *d_pdt,
                             const double *d_u, int64_t nu, const int64_t *d_off);
/* ChemistryIonize::apply; cnt: ncells + 1 + int_scan_blocks(ncells + 1) entries */
void launch_ionize(World &w, const Species &neu, Species &ion, double rate, double dt, const double *d_u,
                   int64_t nu, const int64_t *d_off, int32_t *cnt, uint64_t stream);
void launch_inv_vol(World &w);
void launch_charge(World &w);
void launch_add_fp64(World &w, Species &s, const double *d_pos3, const double *d_vel3,
                     const double *d_w, int64_t n, int rewind);
void launch_load_box(World &w, Species &s, const double x1[3], const double x2[3], double mpw,
                     int64_t num_mp, const double *d_u, uint64_t stream_id);
void launch_load_qs(World &w, Species &s, const double x1[3], const double x2[3], double mpw,
                    const int num_mp[3]);
void launch_load_thermal(World &w, Species &s, const double x1[3], const double x2[3], double mpw,
                         int64_t num_mp, const double vd[3], double temp, const double *d_u, uint64_t stream_id);
void launch_inject(World &w, Species &s, int num_sim, double v_drift, double temp, int vmode,
                   const double *d_u, uint64_t stream_id);
void launch_diag(World &w, Species &s, double *d_out5);
void launch_pe(World &w, double *d_out1);
void launch_update_average(World &w, Species &s);
int launch_sor_box(World &w, int max_it, double tol);
int launch_gs_sphere(World &w, int max_it, double tol);
void launch_qn(World &w);
void launch_node_vol(World &w);
void launch_ef4(World &w);
void launch_fill(World &w, double *x, int64_t n, double v);
void launch_predict(World &w, bool extrapolate);
void launch_snapshot(World &w, double *out);

/* k_mixed.cu */
void launch_push_mixed(World &w, Species &s, bool deposit);
void launch_deposit_mixed(World &w, Species &s);
void launch_to_mixed(World &w, Species &s, const double *P, int64_t stride, int64_t first,
                     int64_t n);
void launch_from_mixed(World &w, Species &s, double *P, int64_t stride, int64_t n);
void launch_sort_mixed(World &w, Species &s);
void launch_diag_mixed(World &w, Species &s, double *d_out5);
void launch_ens_push(cudaStream_t st, bool push, int blocks, int threads, const EnsBox *boxes, const EnsSeg *segs,
                     const int4 *work, int nwork, const float4 *ef4, int32_t *cell, float *off, float *vel,
                     int64_t stride, unsigned long long *acc, int64_t total_nodes, int *err);
void launch_to_mixed_raw(cudaStream_t st, const Geo &g, const double *P, int64_t pstride, int64_t n, int64_t first,
                         int32_t *cell, float *off, float *vel, int64_t stride);
void launch_from_mixed_raw(cudaStream_t st, const Geo &g, const int32_t *cell, const float *off, const float *vel,
                           int64_t stride, int64_t first, int64_t n, double w0, double *P, int64_t pstride);

/* k_pcg.cu */
int launch_newton_pcg(World &w, bool fp32_inner);
int launch_pcg_linear(World &w, bool fp32, const double *b, double *y, double rel_tol, int max_outer);

}  // namespace espic
