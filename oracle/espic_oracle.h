/*
 * espic_oracle.h -- CPU restatement of the electrostatic PIC time step of
 * "Plasma Simulations by Example" (ch2 grounded box, ch3/ver2 sphere, ch4
 * warm-beam injector).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the CUDA
 * path: only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it.  The product library (libespic) never calls it and
 * has no CPU fallback.
 *
 * Parity is pinned: tests/golden/ holds vectors produced by the reference's
 * own CPU code (compiled from its sources by oracle/build_ref.py) and the
 * tests check every function here against them.
 *
 * Conventions
 *  - Node fields are linear arrays in the reference's U order
 *    (ch3/ver2/Field.h:161): u = k*ni*nj + j*ni + i, i fastest.
 *  - Vector node fields (ef) are interleaved [u][3].
 *  - Particles are a structure-of-arrays block P with row stride `stride`:
 *    P[c*stride + p], c = 0..6 for x, y, z, vx, vy, vz, mpw.
 *  - Every expression keeps the reference's operand order; build with
 *    -ffp-contract=off so that no multiply-add is fused.
 */
#ifndef ESPIC_ORACLE_H
#define ESPIC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int ni, nj, nk, pad;
    double x0[3], xm[3], dh[3];
} eo_grid;

/* Physical constants of the reference, Const:: in ch2/World.h:12-21. */
#define EO_EPS_0 8.85418782e-12
#define EO_QE 1.602176565e-19
#define EO_AMU 1.660538921e-27
#define EO_ME 9.10938215e-31
#define EO_K 1.380648e-23
#define EO_PI 3.141592653

/* ---- counter-based RNG (Philox4x32-10, Salmon et al., SC'11) ---------- */
void eo_philox4x32(uint32_t ctr[4], const uint32_t key[2]);
double eo_philox_uniform(uint64_t seed, uint64_t stream, uint64_t index);
void eo_philox_uniforms(uint64_t seed, uint64_t stream, uint64_t first, int64_t n, double *out);

/* ---- geometry: World::setExtents ch2/World.cpp:22-36 ---------------------- */
void eo_grid_set(eo_grid *g, int ni, int nj, int nk, const double x0[3], const double xm[3]);
void eo_node_volumes(const eo_grid *g, double *vol);
void eo_xtol(const eo_grid *g, const double x[3], double lc[3]);
void eo_gather3(const eo_grid *g, const double *ef, const double lc[3], double out[3]);
int eo_in_bounds(const eo_grid *g, const double x[3]);

/* ---- particles ------------------------------------------------------- */
void eo_push_box(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                 double *P, int64_t stride, int64_t n);
int64_t eo_push_sphere(const eo_grid *g, const double *ef, const double sphere[4], double charge,
                       double mass, double dt, double *P, int64_t stride, int64_t n);
int64_t eo_compact_swap_last(double *P, int64_t stride, int64_t n);
int64_t eo_compact_holes(double *P, int64_t stride, int64_t n);
int64_t eo_add_particles(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                         const double *pos3, const double *vel3, const double *w, int64_t n,
                         double *P, int64_t stride, int64_t np0, int64_t cap);
int64_t eo_load_box(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                    const double x1[3], const double x2[3], double num_den, int64_t num_mp,
                    const double *u, double *P, int64_t stride, int64_t np0, int64_t cap);
int64_t eo_load_box_qs(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       const double x1[3], const double x2[3], double num_den, const int num_mp[3],
                       double *P, int64_t stride, int64_t np0, int64_t cap);
int64_t eo_load_box_thermal(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                            const double x1[3], const double x2[3], double mpw, int64_t num_mp,
                            const double vd[3], double temp, const double *u, double *P, int64_t stride,
                            int64_t np0, int64_t cap);
int64_t eo_inject_cold(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       double mpw0, double v_drift, double den, const double *u, int64_t *u_used,
                       double *P, int64_t stride, int64_t np0, int64_t cap);
int64_t eo_inject_warm(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       double mpw0, double v_drift, double den, double temp, const double *u,
                       int64_t *u_used, double *P, int64_t stride, int64_t np0, int64_t cap);
int eo_inject_count(const eo_grid *g, double dt, double mpw0, double v_drift, double den, double u0);
int64_t eo_inject_beam(const eo_grid *g, const double *ef, double charge, double mass, double dt,
                       double mpw0, double v_drift, double den, double temp, int mode, double *rem,
                       const double *u, int64_t *u_used, double *P, int64_t stride, int64_t np0, int64_t cap);

/* ---- collisions: DSMC_MEX, ch4/Collisions.h:51-75, ch4/Collisions.cpp:84-183 ----
 * One DSMC_MEX::apply(dt) on one species (mass, specific weight mpw0) with the
 * VHS parameters c[4] = {d_ref, omega, 2 K T_ref / m_r, Gamma(5/2 - omega)}:
 * particles grouped by World::XtoC in particle order, NTC group counts from
 * *sigma_cr_max, pairs, collision tests and post-collision angles drawn from
 * u[0..nu) in the reference's rnd() order.  *sigma_cr_max becomes the largest
 * sigma*cr tested when a collision happened.  cell_off (n_cells + 1 entries,
 * optional) receives the index of each cell's first uniform.  Returns the
 * number of collisions, -1 when the uniforms run out. */
int64_t eo_dsmc_mex(const eo_grid *g, double mass, double mpw0, double dt, const double c[4],
                    double *sigma_cr_max, double *P, int64_t stride, int64_t n, const double *u, int64_t nu,
                    int64_t *u_used, int64_t *cell_off);

/* ---- deposit --------------------------------------------------------- */
void eo_deposit_fp64(const eo_grid *g, const double *P, int64_t stride, int64_t n, double *acc);
void eo_deposit_fixed(const eo_grid *g, const double *P, int64_t stride, int64_t n, double fx,
                      int64_t *acc);
void eo_divide_volume(int64_t nn, double *den, const double *vol);
void eo_density_from_fixed(int64_t nn, const int64_t *acc, double inv_fx, const double *vol,
                           double *den);
void eo_charge_density(int64_t nn, int ns, const double *charges, const double *dens, double *rho);
int eo_fixed_scale_exponent(double weight_bound, int64_t capacity);

/* ---- field solve ----------------------------------------------------- */
double eo_residual_box(const eo_grid *g, const double *phi, const double *rho);
int eo_sor_box_lex(const eo_grid *g, double *phi, const double *rho, int max_it, double tol,
                   double *l2_out, int *it_out);
int eo_sor_box_rb(const eo_grid *g, double *phi, const double *rho, int max_it, double tol,
                  double *l2_out, int *it_out);
void eo_objects_sphere(const eo_grid *g, const double c[3], double radius, double phi_s,
                       int *obj, double *phi);
void eo_objects_inlet(const eo_grid *g, int *obj, double *phi);
void eo_neumann_targets(const eo_grid *g, const int *obj, int *target);
double eo_residual_sphere(const eo_grid *g, const double *phi, const double *rho, const int *obj,
                          double phi0, double te0, double n0);
int eo_gs_sphere_lex(const eo_grid *g, double *phi, const double *rho, const int *obj, double phi0,
                     double te0, double n0, int max_it, double tol, double *l2_out, int *it_out);
int eo_sor_sphere_rb(const eo_grid *g, double *phi, const double *rho, const int *obj,
                     const int *target, double phi0, double te0, double n0, int max_it, double tol,
                     double *l2_out, int *it_out);
void eo_qn(const eo_grid *g, double *phi, const double *rho, const int *obj, double phi0,
           double te0, double n0);
int eo_newton_pcg(const eo_grid *g, double *phi, const double *rho, const int *obj,
                  const int *target, double phi0, double te0, double n0, int nr_max, double nr_tol,
                  int pcg_max, double pcg_tol, int *nr_it_out, int *pcg_it_out);
int eo_newton_pcg_fb(const eo_grid *g, double *phi, const double *rho, const int *obj,
                     const int *target, double phi0, double te0, double n0, int nr_max, double nr_tol,
                     int pcg_max, double pcg_tol, int gs_max, double gs_tol, int early_stop, int *nr_it_out,
                     int *pcg_it_out, int *gs_it_out);
void eo_efield(const eo_grid *g, const double *phi, double *ef);

/* ---- diagnostics ----------------------------------------------------- */
void eo_species_diag(const double *P, int64_t stride, int64_t n, double mass, double out[5]);
double eo_potential_energy(const eo_grid *g, const double *ef, const double *vol);
void eo_update_average(int64_t nn, double *ave, const double *inst, int samples);
/* ch4 species moments and MCC (ch4/Species.cpp:191-235, ch4/Collisions.cpp:43-80) */
void eo_sample_moments(const eo_grid *g, const double *P, int64_t stride, int64_t n, double *mom);
void eo_gas_properties(const eo_grid *g, double mass, const double *mom, double *vel, double *T);
void eo_compute_mpc(const eo_grid *g, const double *P, int64_t stride, int64_t n, double *mpc);
int64_t eo_mcc_cex(const eo_grid *g, double *P, int64_t stride, int64_t n, const double *den, const double *vel,
                   double dt, const double *u, int64_t nu, int64_t *u_used, int64_t *p_off);
/* ch4 Species::advance of a neutral species with the sphere's diffuse
 * reflection (ch4/Species.cpp:8-100); pdt: per-particle time left */
int64_t eo_advance_ch4_neutral(const eo_grid *g, const double sphere[4], double mass, double dt, double *P,
                               int64_t stride, int64_t n, double *pdt, const double *u, int64_t nu,
                               int64_t *u_used, int64_t *p_off, int holes);
/* ChemistryIonize::apply (ch4/Collisions.cpp:10-31) */
int64_t eo_chemistry_ionize(const eo_grid *g, const double *den_n, const double *rho, const double *ef,
                            double charge, double mass, double mpw0, double rate, double dt, double *Q,
                            int64_t max_new, double *qdt, const double *u, int64_t nu, int64_t *u_used);
int64_t eo_chemistry_ionize_ex(const eo_grid *g, const double *den_n, const double *rho, const double *ef,
                               double charge, double mass, double mpw0, double rate, double dt, double *Q,
                               int64_t max_new, double *qdt, const double *u, int64_t nu, int64_t *u_used,
                               int64_t *cell_off);
int64_t eo_advance_ch4_ion_ex(const eo_grid *g, const double *ef, const double sphere[4], double charge, double mass,
                              double mpw0, double dt, double *P, int64_t stride, int64_t n, double *pdt,
                              double neu_mpw0, double neu_charge, double neu_mass, double sph_mpw0, double sph_charge,
                              double sph_mass, double *Q, int64_t max_new, int32_t *tag, double *qdt, int64_t *n_new,
                              const double *u, int64_t nu, int64_t *u_used, int64_t *p_off, int holes);
/* ch4 Species::advance of a charged species: ions striking the sphere create
 * neutrals and sputtered particles (ch4/Species.cpp:8-91, 103-119) */
int64_t eo_advance_ch4_ion(const eo_grid *g, const double *ef, const double sphere[4], double charge, double mass,
                           double mpw0, double dt, double *P, int64_t stride, int64_t n, double *pdt,
                           double neu_mpw0, double neu_charge, double neu_mass, double sph_mpw0, double sph_charge,
                           double sph_mass, double *Q, int64_t max_new, int32_t *tag, double *qdt, int64_t *n_new,
                           const double *u, int64_t nu, int64_t *u_used);

/* ---- the mixed particle form (the chosen GPU form) -------------------------
 * int32 cell key i | j<<10 | k<<20, float offsets and velocities [3][stride],
 * weight mpw0; the GPU arithmetic restated operation by operation. */
typedef struct {
    int ni, nj, nk;
    float qmdt;    /* (float)(q/m dt) */
    float dtdh[3]; /* (float)(dt/dh) */
    float dh[3];
    float sx[3];   /* (float)(x0 - sphere centre) */
    float r2;      /* (float)(radius^2), < 0 without a sphere */
} eo_mix_args;
void eo_mix_args_set(eo_mix_args *a, const eo_grid *g, double charge, double mass, double dt,
                     const double *sphere);
void eo_ef_to_f32(int64_t nn, const double *ef, float *ef4);
void eo_to_mixed(const eo_grid *g, const double *P, int64_t pstride, int64_t n, int32_t *cell, float *off,
                 float *vel, int64_t stride);
void eo_from_mixed(const eo_grid *g, const int32_t *cell, const float *off, const float *vel, int64_t stride,
                   int64_t n, double mpw0, double *P, int64_t pstride);
void eo_push_mixed(const eo_mix_args *a, const float *ef4, int walls, int32_t *cell, float *off, float *vel,
                   int64_t stride, int64_t n, uint8_t *dead);
int64_t eo_compact_mixed(int32_t *cell, float *off, float *vel, int64_t stride, int64_t n, const uint8_t *dead);
void eo_deposit_mixed(const eo_grid *g, const int32_t *cell, const float *off, int64_t stride, int64_t n,
                      const uint8_t *skip, int64_t *acc);

/* ---- CPU baseline (threaded like ch9/MT) ------------------------------ */
double eo_bench_push_deposit(const eo_grid *g, const double *ef, const double sphere[4],
                             double charge, double mass, double dt, double fx, double *P,
                             int64_t stride, int64_t n, int threads, int steps, int64_t *n_out,
                             int64_t *acc);

#ifdef __cplusplus
}
#endif
#endif
