/*
 * espic.h -- C-ABI of libespic, the GB300-native electrostatic PIC time step
 * of "Plasma Simulations by Example" (ch2 grounded box, ch3/ver2 flow past a
 * sphere, ch4 warm-beam injector).
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes and
 * returns an int status (ESPIC_OK = 0; > 0 not converged; < 0 error).  No
 * C++ exception crosses this boundary.  Host pointers are ordinary host
 * memory; the library owns all device memory of a world.  All work of a
 * world is ordered on one CUDA stream; calls that return values computed on
 * the device synchronise that stream, the others only enqueue work.
 *
 * Each function names the reference interface it replaces (file:line in the
 * reference tree).
 */
#ifndef ESPIC_H
#define ESPIC_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------- */
#define ESPIC_OK 0
#define ESPIC_NOT_CONVERGED 1  /* PotentialSolver::solve returned false */
#define ESPIC_ERR_ARG (-1)     /* bad argument or handle */
#define ESPIC_ERR_CUDA (-2)    /* CUDA runtime error (message in espic_last_error) */
#define ESPIC_ERR_CAPACITY (-3)/* particle buffer full; particles were not added */
#define ESPIC_ERR_NONFINITE (-4) /* NaN or Inf in the potential solve */
#define ESPIC_ERR_FIXED (-5)   /* weight outside the fixed-point deposit range */
#define ESPIC_ERR_STATE (-6)   /* call not valid in this state */

/* particle storage forms */
#define ESPIC_FORM_FP64 0  /* x, v, mpw in float64 (bit-exact with the reference) */
#define ESPIC_FORM_MIXED 1 /* int32 cell + float32 in-cell offset + float32 velocity */

/* wall treatment of a species */
#define ESPIC_WALLS_REFLECT 0 /* ch2/Species.cpp:32-36 one-bounce mirror */
#define ESPIC_WALLS_ABSORB 1  /* ch3/ver2/Species.cpp:28-32 (also absorbed by the sphere) */

/* potential solvers (ch2/PotentialSolver.h:6-23, ch3/ver2/PotentialSolver.h:40) */
#define ESPIC_SOLVER_SOR 0        /* linear Poisson, Dirichlet walls, red-black SOR (ch2) */
#define ESPIC_SOLVER_GS 1         /* Boltzmann electrons, red-black nonlinear SOR (ch3 GS) */
#define ESPIC_SOLVER_PCG 2        /* Boltzmann electrons, Newton + Jacobi-PCG (ch3 PCG) */
#define ESPIC_SOLVER_QN 3         /* quasi-neutral log inversion (ch3 QN) */

/* node fields for espic_field_read / espic_field_write */
#define ESPIC_FIELD_PHI 0
#define ESPIC_FIELD_RHO 1
#define ESPIC_FIELD_NODE_VOL 2
#define ESPIC_FIELD_EF 3      /* 3 values per node, interleaved */
#define ESPIC_FIELD_DEN 4     /* number density of one species */
#define ESPIC_FIELD_DEN_AVE 5 /* running average of den */
#define ESPIC_FIELD_OBJECT_ID 6 /* int32 values travelled as float64 */
/* ch4 species fields (float64 form; ch4/Species.h:84-95) */
#define ESPIC_FIELD_VEL 7     /* stream velocity, 3 values per node, interleaved */
#define ESPIC_FIELD_TEMP 8    /* temperature (K) */
#define ESPIC_FIELD_MPC 9     /* macroparticles per cell, (ni-1)(nj-1)(nk-1) values, i fastest */
#define ESPIC_FIELD_MOMENTS 10 /* sampled sums n, nu, nv, nw, nuu, nvv, nww: 7 planes of nn (read only) */

typedef struct espic_world espic_world;

/* Copies the last error message of the calling thread into buf. */
int espic_last_error(char *buf, int len);

/* ---- World --------------------------------------------------------------- */
/* World::World + World::setExtents, ch2/World.cpp:14-36 (ch3/ver2/World.cpp:14-38).
 * Node volumes are computed for (ni,nj,nk); dh = (xm-x0)/(n-1). */
int espic_world_create(int ni, int nj, int nk, const double x0[3], const double xm[3],
                       espic_world **out);
int espic_world_destroy(espic_world *w);
/* World::setTime, ch2/World.h:66 */
int espic_world_set_time(espic_world *w, double dt, int num_ts);
/* World::advanceTime, ch2/World.h:69: returns 1 while ts <= num_ts, else 0
 * (the reference's loop runs num_ts + 1 iterations). */
int espic_world_advance_time(espic_world *w);
/* World::getTs / getTime */
int espic_world_get_time(espic_world *w, int *ts, double *time);
/* World::addSphere, ch3/ver2/World.cpp:88-106 */
int espic_world_add_sphere(espic_world *w, const double center[3], double radius, double phi_sphere);
/* World::addInlet, ch3/ver2/World.cpp:109-116 */
int espic_world_add_inlet(espic_world *w);
/* Key of the Philox streams behind every random draw of this world (the
 * reference seeds a global mt19937 from std::random_device, ch2/World.h:24-33). */
int espic_world_set_seed(espic_world *w, uint64_t seed);
/* Waits for the world's stream; returns any error flagged on the device. */
int espic_world_sync(espic_world *w);
/* The cudaStream_t (as void*) on which all of the world's work is ordered, so
 * that a caller can record events on it or order its own work after it.  No
 * reference counterpart (the reference has no device stream). */
int espic_world_stream(espic_world *w, void **stream);

/* ---- Species ------------------------------------------------------------- */
/* Species::Species, ch2/Species.h:25-28 (mpw0 = 0) and ch3/ver2/Species.h:25-29.
 * capacity = maximum number of macroparticles kept on the device;
 * weight_bound = largest macroparticle weight the fixed-point deposit must
 * hold (0: use mpw0, or the weight of the first load). */
int espic_species_create(espic_world *w, double mass, double charge, double mpw0, int64_t capacity,
                         int form, int walls, double weight_bound, int *species_id);
/* Species::getNp, ch2/Species.h:31 */
int espic_species_count(espic_world *w, int sp, int64_t *np);
/* Species::addParticle for n particles, ch2/Species.cpp:55-71: particles outside
 * [x0,xm) are rejected; velocities are rewound by (q/m) E dt/2.  pos3/vel3 are
 * [n][3], mpw is [n] (NULL: mpw0). */
int espic_species_add(espic_world *w, int sp, const double *pos3, const double *vel3,
                      const double *mpw, int64_t n);
/* Direct state access through the public Species::particles vector
 * (ch2/Species.h:60): P is [7][stride] = x, y, z, vx, vy, vz, mpw; no rewind.
 * espic_species_set replaces the particles; espic_species_get copies them out
 * (the mixed form is converted to float64). */
int espic_species_set(espic_world *w, int sp, const double *P, int64_t stride, int64_t n);
int espic_species_get(espic_world *w, int sp, double *P, int64_t stride, int64_t cap, int64_t *n);
/* The same access to Species::particles (ch2/Species.h:60) for a species in
 * the mixed form, without conversion: cell keys i | j<<10 | k<<20 ([n]),
 * in-cell offsets and velocities ([3][stride] float).  The state round-trips
 * bit for bit (checkpoints, parity checks of the mixed arithmetic).
 * espic_species_set_mixed refuses keys outside the cells and offsets outside
 * [0,1] with ESPIC_ERR_ARG before copying anything. */
int espic_species_set_mixed(espic_world *w, int sp, const int32_t *cell, const float *off, const float *vel,
                            int64_t stride, int64_t n);
int espic_species_get_mixed(espic_world *w, int sp, int32_t *cell, float *off, float *vel, int64_t stride,
                            int64_t cap, int64_t *n);
/* Species::loadParticlesBox, ch2/Species.cpp:74-97.  u = 3*num_mp uniforms
 * (x, y, z per particle) or NULL to draw them from the world's Philox stream. */
int espic_species_load_box(espic_world *w, int sp, const double x1[3], const double x2[3],
                           double num_den, int64_t num_mp, const double *u);
/* loadParticlesBox with velocities: num_mp particles of weight mpw (0: the
 * species' mpw0), uniform in the box, velocities a drifting Maxwellian of
 * temperature temp (K) about v_drift, sampled by Box-Muller; rewound by half
 * a step like addParticle.  No single reference counterpart (closest:
 * Species::sampleIsotropicVel, ch4/Species.cpp:161-175).  u = 7 uniforms per
 * particle (x, y, z, then 4 for the normals) or NULL for the world's Philox
 * stream.  Used to set up steady-state-like initial states. */
int espic_species_load_box_thermal(espic_world *w, int sp, const double x1[3], const double x2[3],
                                   double mpw, int64_t num_mp, const double v_drift[3], double temp,
                                   const double *u);
/* Species::loadParticlesBoxQS, ch2/Species.cpp:101-141 */
int espic_species_load_box_qs(espic_world *w, int sp, const double x1[3], const double x2[3],
                              double num_den, const int num_mp[3]);

/* ---- the time step ------------------------------------------------------- */
/* Species::advance, ch2/Species.cpp:7-38 (reflect) or ch3/ver2/Species.cpp:7-48
 * (absorb + removal).  With deposit != 0 the push also performs
 * Species::computeNumberDensity (ch2/Species.cpp:41-52) on the moved particles. */
int espic_push(espic_world *w, int sp, int deposit);
/* Species::computeNumberDensity, ch2/Species.cpp:41-52 (fixed-point deposit). */
int espic_deposit(espic_world *w, int sp);
/* World::computeChargeDensity, ch2/World.cpp:46-54 */
int espic_charge_density(espic_world *w);
/* counting sort of a species by cell (mixed form; no-op for float64) */
int espic_sort(espic_world *w, int sp);
/* ColdBeamSource (ch3/ver2/Source.h:8-21; temp = 0) and WarmBeamSource
 * (ch4/Source.h:32-46; temp in K) on the z = x0 face. */
int espic_source_create(espic_world *w, int sp, double v_drift, double den, double temp,
                        int *source_id);
/* Velocity and count modes of a source.  Velocity: ESPIC_BEAM_COLD (v_drift
 * along z, ColdBeamSource, ch3/ver2/Source.cpp:4-27), ESPIC_BEAM_WARM (the
 * ch4 approximation, sampleIsotropicVel x sampleVth, ch4/Species.cpp:149-175;
 * the default when temp > 0), ESPIC_BEAM_ISOTROPIC (ch9/MPI/src/Source.cpp:
 * 39-59: isotropic direction at the speed sqrt(2 kT/m), drift added, v_z < 0
 * reflected) and ESPIC_BEAM_MAXWELLIAN (normal components of deviation
 * sqrt(kT/m) by Box-Muller, drift added, v_z < 0 reflected).  Count:
 * ESPIC_COUNT_RANDOM ((int)(N/mpw0 + U), ch3/ver2/Source.cpp:18) or
 * ESPIC_COUNT_REMAINDER ((int)(N/mpw0 + r), the fraction r carried to the next
 * sample, ch9/MPI/src/Source.cpp:20-27).  Explicit uniforms
 * (espic_source_sample_uniforms): one count slot (unused by the remainder
 * count), then 2 / 13 / 4 / 6 per particle for the four velocity modes. */
#define ESPIC_BEAM_COLD 0
#define ESPIC_BEAM_WARM 1
#define ESPIC_BEAM_ISOTROPIC 2
#define ESPIC_BEAM_MAXWELLIAN 3
#define ESPIC_COUNT_RANDOM 0
#define ESPIC_COUNT_REMAINDER 1
int espic_source_set_mode(espic_world *w, int source, int velocity_mode, int count_mode);
/* ColdBeamSource::sample / WarmBeamSource::sample, ch3/ver2/Source.cpp:4-27,
 * ch4/Source.cpp:31-55, drawing from the world's Philox stream. */
int espic_source_sample(espic_world *w, int source);
/* The same with the uniforms given (the reference's order: the count draw,
 * then 2 per particle for a cold source, 13 per particle for a warm one);
 * *used receives the number consumed. */
int espic_source_sample_uniforms(espic_world *w, int source, const double *u, int64_t nu,
                                 int64_t *used);

/* PotentialSolver constructor arguments: ch2/PotentialSolver.h:9-10
 * (max_it, tol) and ch3/ver2/PotentialSolver.h:46-50 (type, max_it, tol). */
int espic_solver_set(espic_world *w, int kind, int max_it, double tol);
/* PotentialSolver::setReferenceValues(phi0, Te0, n0), ch3/ver2/PotentialSolver.h:53-57 */
int espic_solver_set_reference(espic_world *w, double phi0, double te0, double n0);
/* Newton-PCG controls: at most nr_max Newton steps, stop when RMS(update) <
 * nr_tol (ch3/ver2/PotentialSolver.cpp:228-229); inner PCG stops at
 * |r| <= pcg_tol |F|; fp32_inner = 1 runs the PCG in float32 under the
 * float64 Newton residual (iterative refinement). */
int espic_solver_set_newton(espic_world *w, int nr_max, double nr_tol, int pcg_max,
                            double pcg_tol, int fp32_inner);
/* Preconditioner of the Newton-PCG inner solve: levels = number of
 * aggregation-multigrid levels below the node grid (0: Jacobi, as the
 * reference's solvePCGLinear, ch3/ver2/PotentialSolver.cpp:299-331; the
 * default 12 means as many as the grid allows), scale = coarse-correction
 * scale (default 1.6). */
int espic_solver_set_multigrid(espic_world *w, int levels, double scale);
/* Upper bound on the thread blocks of the cooperative solver launches
 * (0: one per SM).  A tuning knob with no reference counterpart: small grids
 * are bound by grid-barrier latency, which falls with fewer blocks. */
int espic_solver_set_launch(espic_world *w, int max_blocks);
/* Newton predictor (default on): when exactly one charge density was
 * computed since the last solve (consecutive steps), the Newton-PCG solve
 * starts on the unknowns from 2 phi^n - phi^(n-1) instead of phi^n, and the
 * float-inner solve, once the solve before was consecutive too, from
 * 3 phi^n - 3 phi^(n-1) + phi^(n-2); the converged solution and its test
 * are unchanged.  No reference counterpart (the reference starts from
 * phi^n). */
int espic_solver_set_predictor(espic_world *w, int enable);
/* The reference's fallback when the inner linear PCG fails
 * (ch3/ver2/PotentialSolver.cpp:270-271): Gauss-Seidel with omega 1
 * (solveGSLinear, :433-461) on the same linear system from the PCG's last
 * iterate, up to the solver's max_it sweeps, residual RMS checked every 25
 * sweeps against its tolerance.  On (1) by default; 0 turns it off. */
int espic_solver_set_fallback(espic_world *w, int enable);
/* The last solve's outcome (waits for the world's stream): converged flag,
 * Newton (or SOR/GS) iterations, inner PCG iterations, fallback Gauss-Seidel
 * sweeps and the final norm. */
int espic_solver_status(espic_world *w, int *converged, int *iterations, int *inner_iterations,
                        int *fallback_sweeps, double *residual);
/* Multigrid levels with fewer than block_nodes nodes run on one thread block
 * between two grid barriers (default 4096); larger levels run on the whole
 * grid.  A tuning knob with no reference counterpart. */
int espic_solver_set_coarse(espic_world *w, int64_t block_nodes);
/* The first multigrid level with at most max_nodes nodes (<= 4096; default
 * 1024) becomes the coarsest and is solved by its dense inverse, computed
 * once per geometry; 0 keeps smoothing sweeps on the coarsest level.  A
 * tuning knob with no reference counterpart. */
int espic_solver_set_dense(espic_world *w, int64_t max_nodes);
/* PotentialSolver::solve, ch2/PotentialSolver.cpp:11-67 and
 * ch3/ver2/PotentialSolver.h:66-75.  With all out-pointers NULL the solve is
 * only enqueued; otherwise the call waits and reports iterations and the
 * final residual.  Returns ESPIC_NOT_CONVERGED when the reference's solve
 * would return false. */
int espic_solve(espic_world *w, int *iterations, int *inner_iterations, double *residual);
/* PotentialSolver::computeEF, ch2/PotentialSolver.cpp:70-110 */
int espic_efield(espic_world *w);

/* ---- diagnostics ----------------------------------------------------------- */
/* Species::getRealCount, getMomentum, getKE, ch2/Species.cpp:144-168:
 * out = {real count, px, py, pz, KE} */
int espic_species_diag(espic_world *w, int sp, double out[5]);

/* DSMC_MEX, ch4/Collisions.h:51-75 and ch4/Collisions.cpp:84-183:
 * neutral-neutral collisions of a species in the float64 form by Bird's
 * no-time-counter scheme with the variable-hard-sphere cross-section.
 * c = {d_ref, omega, 2 K T_ref / m_r, Gamma(5/2 - omega)}, or NULL for the
 * reference's constructor values (d_ref 4.07e-10 m, omega 0.77, T_ref
 * 273.15 K); sigma_cr_max is the member's starting value (1e-14 in the
 * reference).  DSMC_MEX::apply(dt) is espic_dsmc_apply with u NULL: each
 * cell draws its uniforms from the world's counter-based stream.  With u
 * non-NULL (parity checks) cell c draws u[cell_off[c]], u[cell_off[c] + 1],
 * ... in the reference's rnd() order (cell_off: n_cells + 1 entries); the
 * call then waits.  espic_dsmc_status reads sigma_cr_max and the collision
 * counts of the last call and of all calls. */
int espic_dsmc_enable(espic_world *w, int sp, const double *c, double sigma_cr_max);
int espic_dsmc_apply(espic_world *w, int sp, double dt, const double *u, int64_t nu, const int64_t *cell_off);
int espic_dsmc_status(espic_world *w, int sp, double *sigma_cr_max, int64_t *collisions_last,
                      int64_t *collisions_total);
/* Species::sampleMoments (ch4/Species.cpp:191-201): adds each particle's
 * mpw, mpw v and mpw v_d v_d to the sampled sums with the CIC corner weights
 * of Field_::scatter.  Each corner product is rounded to a 64-bit integer
 * count of 2^-S (S per sum and call, from the call's largest value, so no
 * node overflows) and summed exactly: deterministic, within ~1e-13 relative
 * of the reference's float64 sums. */
int espic_sample_moments(espic_world *w, int sp);
/* Species::computeGasProperties (ch4/Species.cpp:204-225): ESPIC_FIELD_VEL
 * and ESPIC_FIELD_TEMP from the sampled sums */
int espic_gas_properties(espic_world *w, int sp);
/* Species::clearSamples (ch4/Species.cpp:238-240) */
int espic_clear_samples(espic_world *w, int sp);
/* Species::computeMPC (ch4/Species.cpp:228-235): ESPIC_FIELD_MPC */
int espic_compute_mpc(espic_world *w, int sp);
/* MCC_CEX(source, target).apply(dt) (ch4/Collisions.h:40-50,
 * ch4/Collisions.cpp:43-80): each source particle collides with the target
 * gas (den and ESPIC_FIELD_VEL of species tgt, gathered at the particle)
 * with probability 1 - exp(-n sigma |v - v_t| dt), sigma = 1e-16 m^2, and a
 * colliding particle's velocity is set to 0, as in the reference.  u NULL:
 * particle p draws index p of the call's counter-based stream.  u non-NULL
 * (parity checks): particle p draws u[p_off[p]] (p_off: one entry per
 * particle) and the call waits.  collisions (may be NULL; non-NULL waits):
 * the number of colliding particles. */
int espic_mcc_cex(espic_world *w, int src, int tgt, double dt, const double *u, int64_t nu, const int64_t *p_off,
                  int64_t *collisions);
/* Species::advance(neutrals, spherium) of a species of charge 0
 * (ch4/Species.cpp:8-100) with the world's dt: each particle moves for its
 * time left plus dt; leaving the domain removes it; striking the sphere
 * re-emits it diffusely at the speed of a 1000 K wall and it moves on for the
 * time it had used (the reference's arithmetic).  pdt NULL: particles
 * appended since the last call (sources, loaders, espic_species_set) have
 * one dt left, as addParticle leaves them (ch4/Species.h:65), the others
 * none; pdt non-NULL: each particle's time left (one per particle).  u NULL:
 * particle p draws from the call's counter-based stream; u non-NULL (parity
 * checks): particle p's k-th uniform is u[p_off[p] + k], 11 per bounce.  The
 * removal keeps this library's compaction order (the survivors of the
 * reference's swap-with-last).  bounces (may be NULL; non-NULL waits): sphere
 * strikes of the call.  Charged species move with espic_advance_ch4_ions. */
int espic_advance_ch4(espic_world *w, int sp, const double *pdt, const double *u, int64_t nu, const int64_t *p_off,
                      int64_t *bounces);
/* Species::advance(neutrals, spherium) of a charged species (ch4's ion
 * branch, ch4/Species.cpp:8-91) with the world's dt: each ion's velocity is
 * kicked by E (t q / m) over its time left t (plus dt), then it moves for t;
 * leaving the domain removes it; striking the sphere removes it and adds,
 * at 0.999 of the way to the surface, (int)(mpw0 / neutrals' mpw0 + U)
 * particles to species `neutrals` and, above 5000 m/s, (int)(0.1 mpw0 /
 * spherium's mpw0 + U) to species `spherium` (which may be `neutrals`), each
 * with a diffusely reflected velocity at the speed of a 1000 K wall for the
 * ion's mass, rewound by the target's q/m E dt/2, the target's mpw0 and one
 * dt of time left (Species::addParticle, ch4/Species.cpp:103-119).  Each
 * target receives the particles in ion order (an ion's neutrals before its
 * sputtered particles).  pdt, u, p_off as espic_advance_ch4, u holding per
 * strike the neutral count's uniform, 11 per neutral, the sputter count's,
 * 11 per sputtered particle.  The targets must be other float64-form
 * species.  The call waits.  strikes (may be NULL): ions that struck the
 * sphere. */
int espic_advance_ch4_ions(espic_world *w, int sp, int neutrals, int spherium, const double *pdt, const double *u,
                           int64_t nu, const int64_t *p_off, int64_t *strikes);
/* ChemistryIonize(neutrals, ions, rate).apply(dt), ch4/Collisions.cpp:10-31:
 * for each cell (the reference's order: i outer, k inner), n_a (neutrals'
 * den) and n_e = rho / QE at the cell centre, and (int)(rate n_a n_e dt dV /
 * ions' mpw0 + U) ions added at the cell's corner node (i, j, k) (World::pos
 * of the truncated coordinates, ch4/World.h:107-111) with velocity 0 rewound
 * by q/m E dt/2 and weight mpw0.  They join the species as appended
 * particles (one dt of time left at its next ch4 push; the reference passes
 * mpw0 as addParticle's time-left argument).  u NULL: cell c draws index c of
 * the call's counter-based stream; u non-NULL (parity checks): cell c draws
 * u[cell_off[c]] (cell_off: one entry per cell).  The ion species must be
 * in the float64 form.  The call waits.  created (may be NULL): ions added. */
int espic_chemistry_ionize(espic_world *w, int neutrals, int ions, double rate, double dt, const double *u,
                           int64_t nu, const int64_t *cell_off, int64_t *created);
/* World::getPE, ch2/World.cpp:72-84 */
int espic_potential_energy(espic_world *w, double *pe);
/* The per-step columns of Output::diagOutput, ch3/ver2/Output.cpp:96-132, with
 * one device round trip: for each species {np, real count, px, py, pz, KE},
 * then PE.  row must hold 6*ns + 1 values. */
int espic_diag_row(espic_world *w, double *row, int len);
/* Species::updateAverages / Field_::updateAverage, ch3/ver2/Field.h:214-220 */
int espic_update_average(espic_world *w, int sp);
/* World::steadyState, ch3/ver2/World.cpp:129-158 */
int espic_steady_state(espic_world *w, int *steady);

/* ---- node fields ------------------------------------------------------------ */
/* Host mirrors of World::phi/rho/node_vol/ef/object_id and Species::den/den_ave
 * (the device copy is authoritative, as updateHostPhi in
 * ch9/CUDA/PotentialSolver.cu:323-328).  n = number of float64 values. */
int espic_field_read(espic_world *w, int field, int sp, double *host, int64_t n);
int espic_field_write(espic_world *w, int field, int sp, const double *host, int64_t n);

/* ---- measurement -------------------------------------------------------------- */
/* phases timed by espic_profile (CUDA events on the world's stream) */
#define ESPIC_PHASE_INJECT 0  /* source sampling and loads */
#define ESPIC_PHASE_SORT 1    /* counting sort by cell */
#define ESPIC_PHASE_PUSH 2    /* the push kernel (with its fused deposit) */
#define ESPIC_PHASE_COMPACT 3 /* removal of absorbed particles */
#define ESPIC_PHASE_DENSITY 4 /* accumulator clear, density and charge density */
#define ESPIC_PHASE_SOLVE 5   /* potential solve */
#define ESPIC_PHASE_EFIELD 6  /* computeEF */
#define ESPIC_PHASE_DIAG 7    /* diagnostics reductions */
#define ESPIC_NPHASES 8
/* Turns per-phase event timing on (1) or off (0); turning it on clears the
 * totals.  The reference only records wall time per step
 * (ch2/World.cpp:39-43, ch2/Output.cpp:99). */
int espic_profile(espic_world *w, int enable);
/* Waits for the world's stream and returns, per phase, the summed device
 * milliseconds and the number of timed ranges; *launches receives the number
 * of kernels launched on this world so far. */
int espic_profile_read(espic_world *w, double ms[ESPIC_NPHASES], int64_t count[ESPIC_NPHASES],
                       int64_t *launches);
/* Totals over all solves so far: Newton (or SOR) iterations and inner PCG
 * iterations, summed on the device. */
int espic_solver_totals(espic_world *w, int64_t *solves, int64_t *outer, int64_t *inner);

/* ---- deposit without allocation --------------------------------------------- */
/* A library entry point with no counterpart in the reference.  It exists for
 * callers that may not allocate device memory once they are running: a host
 * application or plugin host that has already given all device memory to its
 * own pool allocator, a loop with real-time deadlines that forbids allocation
 * after start-up, or code that must not synchronise the device, which
 * cudaMalloc and cudaFree may do.  It computes the CIC number density of
 * espic_deposit (same corner order, same rounding of each corner weight to a
 * count of 1/fx, same division by the node volume) from particles the caller
 * already holds on the device: d_P is [7][stride] float64 (x, y, z, vx, vy,
 * vz, mpw; only x, y, z and mpw are read), d_den receives ni*nj*nk values in
 * U order.  The fixed-point scale fx is that of a species of capacity n whose
 * weights do not exceed weight_bound, so the result equals espic_deposit's bit
 * for bit when that species' capacity is n.
 *
 * It allocates nothing: its int64 scratch is a static device array of
 * ESPIC_NOALLOC_MAX_NODES nodes (8 MiB, held by every GPU that loads the
 * library until the process exits), and a larger grid is refused with
 * ESPIC_ERR_ARG before any work.  The first call on a device looks up that
 * array's device address (no allocation, but make this first call before any
 * stream capture).  Work is queued on `stream` (a cudaStream_t; NULL for the
 * default stream) and the call returns without waiting.  Every call shares the
 * one scratch array and clears the part it uses before use; calls whose work
 * overlaps on the GPU (other streams, other threads) race on it and must be
 * serialised by the caller.
 *
 * d_flags (optional, a caller-owned device int) is set to 0 on the stream and
 * then receives ESPIC_NOALLOC_RANGE for a weight with |mpw| > weight_bound and
 * ESPIC_NOALLOC_NONFINITE for a non-finite position; such particles deposit
 * nothing.  Read it after the stream's work has finished. */
#define ESPIC_NOALLOC_MAX_NODES (1 << 20)
#define ESPIC_NOALLOC_RANGE 1
#define ESPIC_NOALLOC_NONFINITE 2
int espic_deposit_noalloc(const double *d_P, int64_t stride, int64_t n, int ni, int nj, int nk,
                          const double x0[3], const double xm[3], double weight_bound, double *d_den,
                          int *d_flags, void *stream);

/* ---- output snapshots ------------------------------------------------------- */
/* Output::fields (ch3/ver2/Output.cpp:12-79) without stalling the step: packs
 * the node fields of the VTK file -- object_id, node_vol, phi, rho, then den
 * and den_ave of every species, then ef ([nn][3]) -- into a device buffer on
 * the world's stream (so later steps do not change it) and copies them to
 * pinned host memory on a second stream; returns a ticket at once.  Two
 * snapshots can be in flight; a third reuses the oldest slot after its copy
 * has finished. */
int espic_snapshot_begin(espic_world *w, int64_t *ticket);
/* waits for snapshot `ticket`; *host points at its (7 + 2 * nspecies) * nn
 * doubles in the order above, valid until the slot is reused by the
 * snapshot two tickets later.  May be called from another host thread. */
int espic_snapshot_wait(espic_world *w, int64_t ticket, const double **host, int64_t *count);

/* ---- one whole step --------------------------------------------------------- */
/* One iteration of the ch3/ver2/Main.cpp:50-72 loop body: sample every
 * source, push + deposit every species (sorting mixed species every
 * sort_every steps), charge density, solve, computeEF.  When row != NULL the
 * diag row of espic_diag_row is also returned (one synchronisation). */
int espic_step(espic_world *w, int sort_every, double *row, int len);

/* ---- batched ensemble of independent boxes ------------------------------ */
/* No single reference interface: an ensemble is many ch2 grounded boxes
 * (ch2/Main.cpp:14-75: World, two Species with reflecting walls, the SOR
 * PotentialSolver) stepped together.  Every box has its own node counts and
 * extents; every (box, species) its own weight mpw0 and capacity.  Particles
 * are in the mixed form.  A step runs push + deposit of all boxes in one
 * launch over a flattened work list, then one launch in which clusters of
 * thread blocks claim boxes and compute charge density, red-black SOR
 * (float32 sweeps under a float64 residual, ch2/PotentialSolver.cpp:11-67
 * convergence test) and E;
 * espic_ensemble_step replays the step as a captured CUDA graph. */
typedef struct espic_ensemble espic_ensemble;
/* nodes[3*b..], x0[3*b..], xm[3*b..] per box; mass[s], charge[s] per species;
 * mpw0[b*nspecies + s] and capacity[b*nspecies + s] per box and species */
int espic_ensemble_create(int nbox, const int32_t *nodes, const double *x0, const double *xm, int nspecies,
                          const double *mass, const double *charge, const double *mpw0, const int64_t *capacity,
                          double dt, espic_ensemble **out);
void espic_ensemble_destroy(espic_ensemble *e);
/* Sharding an ensemble over GPUs (one process per GPU, no exchange: the
 * boxes are independent).  espic_partition_boxes assigns nbox boxes of the
 * given work to nparts parts (largest work first, each to the least loaded
 * part; deterministic, so every rank computes the same owner[]); load
 * (optional, [nparts]) receives each part's work.  espic_ensemble_set_box_ids
 * gives the boxes of a part their ids in the whole ensemble, which key their
 * random streams, so a box loads the same particles on whichever rank owns
 * it (ids NULL: the box index).  The ch9/MPI decomposition
 * (ch9/MPI/include/World.h:73-128) splits one domain; boxes need no split. */
int espic_partition_boxes(int nbox, const double *work, int nparts, int32_t *owner, double *load);
int espic_ensemble_set_box_ids(espic_ensemble *e, const int32_t *ids);
int espic_ensemble_set_seed(espic_ensemble *e, uint64_t seed);
/* particles of (box, species) from a host [7][stride] float64 block (replaces
 * the segment); the weight row is ignored (the segment's mpw0 is used) */
int espic_ensemble_set_particles(espic_ensemble *e, int box, int sp, const double *P, int64_t stride, int64_t n);
/* P = NULL returns the count only */
int espic_ensemble_get_particles(espic_ensemble *e, int box, int sp, double *P, int64_t stride, int64_t cap,
                                 int64_t *n);
/* Species::loadParticlesBox (ch2/Species.cpp:74-97) on the GPU: num_mp
 * particles uniform in [x1, x2) from the ensemble's Philox stream, v = 0 */
int espic_ensemble_load_box(espic_ensemble *e, int box, int sp, const double x1[3], const double x2[3],
                            int64_t num_mp);
/* SOR controls shared by every box; omega = 0 selects each box's optimal
 * red-black factor (Young), omega in (0, 2) is used as given (the reference
 * hard-codes 1.4) */
int espic_ensemble_set_solver(espic_ensemble *e, int max_it, double tol, double omega);
/* launch shape: particles per work item (>= 256), push block (128/256/512),
 * solve block (256/512/1024), CTAs per box cluster (1/2/4/8); results do
 * not depend on it */
int espic_ensemble_set_launch(espic_ensemble *e, int chunk, int push_threads, int solve_threads, int cluster);
int espic_ensemble_get_launch(espic_ensemble *e, int *chunk, int *push_threads, int *solve_threads, int *cluster);
/* times every launch shape on real steps and keeps the fastest (consumes 27
 * steps of the run; results do not depend on the shape) */
int espic_ensemble_autotune(espic_ensemble *e, int *chunk, int *push_threads, int *solve_threads, double *push_ms,
                            double *solve_ms);
/* deposit, charge density, solve and E: the state before the first step */
int espic_ensemble_prepare(espic_ensemble *e);
/* nsteps steps through the captured step graph (asynchronous) */
int espic_ensemble_step(espic_ensemble *e, int nsteps);
/* the same steps as direct launches */
int espic_ensemble_step_direct(espic_ensemble *e, int nsteps);
int espic_ensemble_sync(espic_ensemble *e);
void *espic_ensemble_stream(espic_ensemble *e);
int espic_ensemble_launches(espic_ensemble *e, int64_t *n);
int espic_ensemble_steps_taken(espic_ensemble *e, int64_t *steps);
/* per box: sweeps and convergence of the last solve, its float64 residual */
int espic_ensemble_status(espic_ensemble *e, int32_t *sweeps, int32_t *converged, double *residual);
/* ESPIC_FIELD_PHI, _RHO, _EF ([nn][3]) or _DEN (of species sp) of one box */
int espic_ensemble_read(espic_ensemble *e, int box, int field, int sp, double *out);
/* out[b*(nspecies+1) + s]: kinetic energy of species s, out[b*(nspecies+1) +
 * nspecies]: field energy (getKE, ch2/Species.cpp:144-168; getPE,
 * ch2/World.cpp:72-84) */
int espic_ensemble_diag(espic_ensemble *e, double *out);

/* ---- differentiable sphere run --------------------------------------------- */
/* No reference counterpart.  One ion species in a World that has its sphere
 * and inlet and Boltzmann reference values set (the Newton-PCG controls of
 * espic_solver_set_newton apply), stepped without injection.  Absorption is
 * the C1 factor of an absorbing layer of thickness delta just inside the
 * sphere and every face (delta -> 0 is the reference's removal,
 * ch3/ver2/Species.cpp:26-33).  Loss = alpha * field energy of the final
 * potential (World::getPE, ch2/World.cpp:72-84) + beta * ions in the wake
 * box (nodes with z in [wake_z0, wake_z1], CIC weights).  Gradients come from
 * hand-written adjoint kernels of push, gather, deposit, E stencil and solve
 * (the adjoint solve is the Newton-PCG kernel in linear mode), with
 * checkpoints every checkpoint_every steps and recompute.  precision 0:
 * float64 particles and adjoints, 1: float32 (solves keep float64 outer
 * iterations). */
typedef struct espic_diff espic_diff;
int espic_diff_create(espic_world *w, int precision, double mass, double charge, double mpw0, int64_t n,
                      double delta, double wake_z0, double wake_z1, double alpha, double beta,
                      int checkpoint_every, espic_diff **out);
void espic_diff_destroy(espic_diff *d);
/* initial positions x[3][n] and velocities v[3][n] */
int espic_diff_set_state(espic_diff *d, const double *x, const double *v);
/* nsteps steps with the sphere at phi_sphere; *loss receives the loss */
int espic_diff_forward(espic_diff *d, double phi_sphere, int nsteps, double *loss);
/* gradients of the last forward's loss with respect to phi_sphere, x[3][n]
 * and v[3][n] (NULL to skip one) */
int espic_diff_backward(espic_diff *d, double *dloss_dphi_sphere, double *dloss_dx, double *dloss_dv);

#ifdef __cplusplus
}
#endif
#endif
