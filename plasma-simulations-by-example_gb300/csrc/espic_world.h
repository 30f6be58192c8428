/*
 * espic_world.h -- host-side records of a World and its Species (device
 * pointers plus the scalars the launchers need).  Internal to libespic.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <vector>

#include "espic_internal.h"

namespace espic {

struct Species {
    int id = 0;
    int form = 0;   /* ESPIC_FORM_* */
    int walls = 0;  /* ESPIC_WALLS_* */
    double mass = 0, charge = 0, mpw0 = 0;
    bool uniform_w = true; /* every particle carries mpw0: the weight row is not read */
    int64_t cap = 0;
    int64_t ms = 0; /* mixed form: row stride of cell/off/vel, cap rounded up to 64, so every row
                       starts 256-byte aligned for bulk copies */
    /* float64 form: [7][cap] */
    double *P = nullptr;
    /* mixed form */
    int32_t *cell = nullptr, *cell2 = nullptr;
    float *off = nullptr, *off2 = nullptr; /* [3][ms] */
    float *vel = nullptr, *vel2 = nullptr; /* [3][ms] */
    int32_t *sort_count = nullptr;         /* [tile-major cell slots + 1], then the scan's block sums */
    int32_t *seg = nullptr;                /* [ntiles + 1] first particle of each tile after the last sort */
    bool tiled = false;                    /* seg describes the particle order (a sort and no reorder since) */
    /* mixed form: per-block sums (count, v, |v|^2) of the particles the last
     * tile push left, valid until the particles next change */
    double *dsum = nullptr;
    int64_t dsum_cap = 0, dsum_n = 0;
    bool dsum_valid = false;
    /* compaction */
    uint32_t *deadmask = nullptr; /* [cap/32 + 1] */
    int32_t *tiledead = nullptr;  /* [ntiles + 1] */
    int32_t *tilepre = nullptr;   /* [ntiles + 1] exclusive prefix */
    int32_t *holes = nullptr;     /* [cap] */
    int64_t ntiles = 0;
    int64_t *d_count = nullptr; /* device particle count; [1] = count before compaction */
    int64_t host_bound = 0;     /* an upper bound of *d_count known without syncing */
    /* deposit */
    unsigned long long *acc = nullptr; /* [nn] int64 two's complement */
    double *den = nullptr, *den_ave = nullptr;
    int ave_samples = 0;
    double fx = 1.0;      /* float64 form: quantum 1/fx (fx = 2^S) of real particles */
    double unit = 1.0;    /* real particles per accumulator count: 1/fx or mpw0*2^-24 */
    double weight_bound = 0;
    bool deposit_valid = false;
    /* DSMC_MEX collisions (float64 form) */
    bool dsmc_on = false;
    double dsmc_c[4] = {0, 0, 0, 0}; /* VHS: d_ref, omega, 2 K T_ref / m_r, Gamma(5/2 - omega) */
    uint64_t dsmc_calls = 0;
    unsigned long long *d_dsmc = nullptr; /* [0] sigma_cr_max (bits), [1] largest sigma*cr of the call
                                             (bits), [2] collisions of the call, [3] all collisions */
    int32_t *dsmc_cell = nullptr, *dsmc_rank = nullptr, *dsmc_perm = nullptr; /* [cap] */
    int32_t *dsmc_count = nullptr, *dsmc_start = nullptr, *dsmc_bsum = nullptr; /* [ncells + 1], scan */
    /* ch4 moments (allocated on first use): sampled sums [NMOM][nn], the
     * call's integer sums, scales, stream velocity [nn][3], temperature,
     * macroparticles per cell [ncells]; MCC: calls and collision count */
    bool ch4_on = false;
    double *mom = nullptr, *mom_scale = nullptr, *gvel = nullptr, *gtemp = nullptr, *mpc = nullptr;
    unsigned long long *mom_acc = nullptr, *mom_bound = nullptr, *mcc_ncol = nullptr;
    uint64_t mcc_calls = 0;
    /* ch4 neutral push: particles below *ch4_settled have used their time
     * (those above were appended since the last push), bounces of the call */
    int64_t *ch4_settled = nullptr;
    unsigned long long *ch4_bounces = nullptr; /* bounces (neutrals) or sphere strikes (ions) of the call */
    uint64_t ch4_calls = 0;
    /* ch4 ion push: per-ion counts of new particles for each target and
     * their scans' block sums; ChemistryIonize into this species: per-cell
     * counts and block sums (both allocated on first use) */
    int32_t *ch4_cnt = nullptr, *ionize_cnt = nullptr;
    uint64_t ionize_calls = 0;
};

struct Source {
    int sp = 0;
    double v_drift = 0, den = 0, temp = 0;
    uint64_t calls = 0;
    int vmode = 0;         /* ESPIC_BEAM_*: cold, ch4 warm, ch9 isotropic, Maxwellian */
    int count_mode = 0;    /* ESPIC_COUNT_*: random, remainder */
    double remainder = 0;  /* carried fraction of a macroparticle (remainder count) */
};

/* uniforms a beam particle consumes, by velocity mode */
__host__ __device__ inline int beam_uniforms(int vmode) { return vmode == 1 ? 13 : (vmode == 2 ? 4 : (vmode == 3 ? 6 : 2)); }

struct World {
    Geo g{};
    int64_t nn = 0;
    double dt = 0, time = 0;
    int num_ts = 0, ts = -1;
    cudaStream_t stream = nullptr;
    int device = 0, sm_count = 0;
    double *phi = nullptr, *rho = nullptr, *vol = nullptr, *ef = nullptr;
    double *ivol = nullptr; /* RN(1 / node_vol), 0 where the volume is 0: the density's divisor */
    float4 *ef4 = nullptr;
    bool ef4_valid = false;
    bool ef64_valid = true; /* false after a computeEF that wrote ef4 and only the planes k < 2 of ef */
    double *pe_part = nullptr; /* k_efield4's per-block sums of |E|^2 vol */
    int64_t pe_parts = 0;      /* > 0: those sums describe the current field */
    double *phi_ef = nullptr;  /* the potential k_efield4 read (ef is completed from it) */
    int32_t *obj = nullptr, *target = nullptr;
    bool targets_valid = false;
    double sphere[4] = {0, 0, 0, 0}; /* centre, radius^2 */
    bool has_sphere = false;
    int *d_err = nullptr;
    SolveStatus *d_status = nullptr;
    double *d_partials = nullptr; /* reduction scratch */
    int partial_slots = 0;
    double *d_small = nullptr;    /* small results (diag row) */
    double *h_small = nullptr;    /* pinned mirror */
    double *d_u = nullptr;        /* staging for host-given uniforms */
    int64_t d_u_cap = 0;
    double *d_stage = nullptr;    /* staging for host particles */
    int32_t *d_blockcnt = nullptr; /* per-block counts of an append */
    int64_t blockcnt_cap = 0;
    int64_t d_stage_cap = 0;
    /* solver */
    int solver_kind = 0, max_it = 10000;
    double tol = 1e-4, phi0 = 0, te0 = 1.5, n0 = 1e12;
    int nr_max = 20, pcg_max = 10000, fp32_inner = 0;
    bool gs_fallback = true; /* Gauss-Seidel after an inner PCG that fails (the reference's fallback) */
    double nr_tol = 1e-3, pcg_tol = 1e-6;
    void *pcg_buf = nullptr;
    bool pcg_codes_valid = false;
    int pcg_elem = 0;       /* element size the PCG buffers were laid out for */
    int mg_levels_max = 12; /* multigrid levels of the PCG preconditioner (0: Jacobi) */
    double mg_scale = 1.6;  /* coarse-correction scale */
    int64_t mg_block_nodes = 4096; /* multigrid levels smaller than this run on one block */
    int64_t mg_dense_max = 1024;   /* coarsest level solved by its dense inverse when it has at most this
                                      many nodes (0: smoothing sweeps on block 0) */
    int solver_blocks = 0;  /* cap on cooperative solver blocks (0: occupancy limit) */
    double *phi_prev = nullptr;    /* the potential before the last Newton solve (predictor) */
    bool phi_prev_valid = false;
    bool phi_prev2_valid = false;  /* the second row of phi_prev: the solve before phi_prev's, consecutive */
    bool predictor = true;         /* start the Newton solve from 2 phi^n - phi^(n-1) */
    int predict_mode = 0;          /* for the next float-inner solve: 1 copy phi to phi_prev, 2 also extrapolate */
    int64_t rho_version = 0;       /* charge densities computed so far */
    int64_t solve_rho_version = -1;
    double *lin_y = nullptr;       /* linear (adjoint) mode of the Newton-PCG kernel: solution */
    const double *lin_b = nullptr; /* and right-hand side; null for the Newton solve */
    size_t pcg_bytes = 0;
    uint64_t seed = 0x5eed5eed12345ull;
    uint64_t load_calls = 0;
    int64_t step_count = 0;
    int64_t nlaunch = 0; /* kernels launched on this world's stream */
    /* steady state, ch3/ver2/World.h:137-141 */
    bool steady = false;
    double last_mass = 0, last_mom = 0, last_en = 0;
    std::vector<Species *> species;
    std::vector<Source> sources;
    /* output snapshots: two slots of packed node fields (device and pinned
     * host), copied on their own stream */
    struct Snapshot {
        double *dev = nullptr, *host = nullptr;
        size_t count = 0;
        cudaEvent_t packed = nullptr, copied = nullptr;
        int64_t ticket = -1;
    };
    Snapshot snap[2];
    cudaStream_t snap_stream = nullptr;
    int64_t snap_next = 0;
    /* per-phase event timing */
    bool prof = false;
    std::vector<cudaEvent_t> ev_pool;
    struct Range {
        int phase;
        cudaEvent_t a, b;
    };
    std::vector<Range> ranges;
    double prof_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int64_t prof_n[8] = {0, 0, 0, 0, 0, 0, 0, 0};
};

/* n / d for n < 2^24 without an integer division: the float estimate is
 * within one of the quotient (n is exact in float and 1/d is rounded once),
 * and one remainder test corrects it */
/* x == +-0, tested on the 32-bit halves of its bits: written as a 64-bit
 * test of the bits it compiles to a float64 compare, which issues on this
 * GPU's narrow float64 pipe */
__device__ __forceinline__ bool zero_bits(double x) {
    return (((unsigned int)__double2hiint(x) << 1) | (unsigned int)__double2loint(x)) == 0u;
}

__device__ __forceinline__ uint32_t div_small(uint32_t n, uint32_t d, float inv_d) {
    uint32_t q = __float2uint_rz((float)n * inv_d);
    const int32_t r = (int32_t)(n - q * d);
    if (r < 0) q--;
    else if (r >= (int32_t)d) q++;
    return q;
}

/* the eight cloud-in-cell corner weights of a particle at offsets (fx, fy,
 * fz) in its cell, corners in Field_::gather's order (ch2/Field.h:186-208) */
__device__ __forceinline__ void cic_w(float fx, float fy, float fz, float w[8]) {
    float gx = 1.f - fx, gy = 1.f - fy, gz = 1.f - fz;
    w[0] = gx * gy * gz;
    w[1] = fx * gy * gz;
    w[2] = fx * fy * gz;
    w[3] = gx * fy * gz;
    w[4] = gx * gy * fz;
    w[5] = fx * gy * fz;
    w[6] = fx * fy * fz;
    w[7] = gx * fy * fz;
}

/* trilinear E at the particle: a chain of fused multiply-adds over the
 * corners in Field_::gather's order (ch2/Field.h:186-208), from corner 0 */
__device__ __forceinline__ float3 gather_corners(const float w[8], const float4 e[8]) {
    float3 r = make_float3(__fmul_rn(w[0], e[0].x), __fmul_rn(w[0], e[0].y), __fmul_rn(w[0], e[0].z));
#pragma unroll
    for (int c = 1; c < 8; c++) {
        r.x = __fmaf_rn(w[c], e[c].x, r.x);
        r.y = __fmaf_rn(w[c], e[c].y, r.y);
        r.z = __fmaf_rn(w[c], e[c].z, r.z);
    }
    return r;
}

inline int blocks_for(int64_t n, int threads) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > 0x7fffffff) b = 0x7fffffff;
    return (int)b;
}

}  // namespace espic
