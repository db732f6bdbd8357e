/*
 * plume_gpu.h -- C ABI of the GB300 (sm_103a) SPH particle step.
 *
 * The library replaces, for one process on one GPU, the per-step particle
 * path of the Plume-SPH solver: neighbour search, adaptive smoothing length,
 * momentum/energy with artificial viscosity (+ LANS turbulence and heat
 * terms), density / mass-fraction summation with energy smoothing, the LANS
 * velocity filter, the position update, the time-step reduction and the
 * equation of state.  The host keeps its own input files, particle fields,
 * inlet and ghost-wall conventions and calls these entry points instead of
 * the reference free functions.
 *
 * Conventions
 *   - Every entry point returns an int status: PLUME_OK (0) or a PLUME_E_*
 *     code.  No exception or CUDA error crosses the ABI; the text of the last
 *     error of a context is available from plume_last_error().
 *   - Host arrays are owned by the caller and copied at the call.  Device
 *     buffers are owned by the context.  One context per host thread; each
 *     context owns one CUDA stream.  The library keeps no global state.
 *   - Particle identity is a caller-chosen 64-bit key (the host's TKey
 *     packed into 64 bits).  Downloads are in the library's internal
 *     (cell-sorted) order; the key array says which particle is which.
 *
 * Reference interface each entry point replaces (paths inside the Plume-SPH
 * source tree):
 *   plume_create / plume_destroy     compile-time switches of
 *                                    src/plume/options.h:16-837 and the
 *                                    constants of src/plume/parameters.h,
 *                                    bucket grid of src/plume/dataread.cc:247
 *   plume_upload / plume_append      particle creation in add_air.cc:37,491,
 *                                    add_pressure_ghost.cc:37,
 *                                    add_wall_ghost.cc:45,
 *                                    setup_erupt.cc:44, add_new_erupt :389
 *   plume_set_ghost_state            the state write of apply_bcond
 *                                    (src/plume/bcond.cc:196-226)
 *   plume_step / plume_steps         the hot loop of src/plume/main.cc:217-471
 *                                    (3D) and :676-750 (1D): timestep
 *                                    (timestep.cc:94,139), incrtime
 *                                    (src/datstr/properties.h:71-83),
 *                                    search_neighs_consth (neighs.cc:37),
 *                                    adaptive_sml (neighs.cc:479),
 *                                    mom_engr_update (mom_engr_update.cc:29),
 *                                    smooth_density (density_massfrac.cc:25),
 *                                    smooth_velocity (smooth_velocity.cc:25),
 *                                    update_pos (update_pos.cc:34),
 *                                    update_particles_in_bucket
 *                                    (update_pos.cc:171), ifoutput
 *                                    (properties.h:100-118)
 *   plume_download                   reads of Particle fields
 *                                    (src/datstr/particle.h:27-140)
 *   plume_neighbor_pairs             the per-particle neighbour vectors that
 *                                    search_neighs_consth stores with
 *                                    put_neighs (neighs.cc:135,197)
 */
#ifndef PLUME_GPU_H
#define PLUME_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PLUME_OK              0
#define PLUME_E_INVALID       1  /* bad argument or option                   */
#define PLUME_E_CUDA          2  /* a CUDA runtime call failed                */
#define PLUME_E_NONFINITE     3  /* NaN/Inf density, energy or velocity       */
#define PLUME_E_NONPOSITIVE   4  /* density, kernel normalisation or sound
                                    speed <= 0 (the reference asserts:
                                    density_massfrac.cc:293,
                                    smooth_velocity.cc:139, timestep.cc:126)  */
#define PLUME_E_CAPACITY      5  /* particle count beyond the context's
                                    capacity                                  */
#define PLUME_E_OUTSIDE_GRID  6  /* a particle left the bucket grid           */
#define PLUME_E_BUCKET_FULL   7  /* more than max_per_bucket particles in one
                                    bucket (update_pos.cc:427-454)            */
#define PLUME_E_TIMEOUT       8  /* a bounded device wait gave up             */
#define PLUME_E_NOT_BUILT     9  /* library built without device support      */

/* ---- particle boundary-condition types (particle.h:140-150) ----------- */
#define PLUME_BC_ERUPT        0
#define PLUME_BC_PRESSURE     1
#define PLUME_BC_WALL         2
#define PLUME_BC_NOSAVE_REAL 99
#define PLUME_BC_REAL       100

/* ---- bucket flags (bucket.h:183-214 particles_type / has_involved /
 *      bucket_type) ------------------------------------------------------ */
#define PLUME_BUCKET_ABSORBING 0x1 /* has_involved == 0: a real particle that
                                      moves in is deleted (update_pos.cc:289) */
#define PLUME_BUCKET_MIXED     0x2 /* bucket_type == MIXED: escape test
                                      against the domain faces (bucket.cc:435)*/
#define PLUME_BUCKET_INACTIVE  0x4 /* not active: particles in it are not
                                      re-bucketed (update_pos.cc:203)        */
#define PLUME_BUCKET_UNDERGROUND 0x8  /* bucket_type == UNDERGROUND          */
#define PLUME_BUCKET_PRESS_BC    0x10 /* bucket_type == PRESS_BC (the grid's
                                         outer pressure layer); a bucket with
                                         neither these nor MIXED is OVERGROUND */

/* ---- bucket involvement (Bucket::has_involved, bucket.h:230, 400-415):
 *      bit 0 potentially involved particles, bit 1 involved particles ---- */
#define PLUME_BINV_NONE       0  /* outside the domain (pressure ghosts)       */
#define PLUME_BINV_POTENTIAL  1
#define PLUME_BINV_INVOLVED   2
#define PLUME_BINV_BOTH       3

/* ---- arithmetic of the pair sweeps ------------------------------------ */
#define PLUME_PREC_FP64   0  /* every pair term in FP64                       */
#define PLUME_PREC_MIXED  1  /* FP32 pair arithmetic on cell-relative
                                coordinates with compensated FP32 sums; FP64
                                positions, position/energy update and
                                conservation sums                             */

/* ---- smoothing kernels ------------------------------------------------- */
#define PLUME_KERNEL_GAUSS  0 /* sph_lib.cc:207-253: (1/(sqrt(pi) h))^D
                                 exp(-|s|^2), zero if any |s_k| > 3          */
#define PLUME_KERNEL_M4     1 /* cubic B-spline (Monaghan M4), radial support
                                 2h, used by the Sod / ensemble workloads     */

/* ---- momentum/energy discretisation (USE_GSPH, options.h:136-142) ------ */
#define PLUME_METHOD_SPH   0  /* artificial viscosity (mom_engr_update.cc:29-439) */
#define PLUME_METHOD_GSPH_RCM 2 /* USE_GSPH 2, the random choice method:
                                 GSPH with the interface at s* = (sp - 1/2)
                                 |x_i - x_j| and the HLLC problem sampled at
                                 0.6 (sp - 1/2) |x_i - x_j| against its waves'
                                 positions S dt, sp the Van der Corput number
                                 of the step (Generate_VanderCorput,
                                 sph_lib.cc:2214-2245; HLLC_RP_Solver
                                 sph_lib.cc:1859-1885; Riemann_Solver
                                 :2416-2419)                                  */
#define PLUME_METHOD_GSPH  1  /* Godunov SPH: a Riemann problem per pair
                                 (mom_engr_update.cc:441-1146, SHEAR_VEL_APP 2,
                                 RP_MASS_WEIGHTED 0)                           */

/* ---- GSPH Riemann solver (RIEMANN_SOLVER, options.h:185-192, 586-593) -- */
#define PLUME_RIEMANN_ROE   0 /* Roe_RP_Solver, sph_lib.cc:1694-1750 (3D default) */
#define PLUME_RIEMANN_HLLC  1 /* HLLC_RP_Solver, sph_lib.cc:1753-1908,
                                 HLL_WAVE_SPEED_EVA 0 (1D default)            */
#define PLUME_RIEMANN_HLLC_MY 2 /* HLLC_RP_Solver_my, sph_lib.cc:1912-2088:
                                 HLLC for strong shocks, wave speeds by
                                 PlumeOptions.gsph_wave_speed                 */
#define PLUME_RIEMANN_VANLEER 3 /* VanLeer_RP_Solver, sph_lib.cc:2094-2210:
                                 Van Leer's iterative solver on the
                                 Lagrangian sound speeds (at most
                                 PLUME_VANLEER_MAX_ITER iterations here; a
                                 problem that has not converged by then gives
                                 NaN, which the step reports)                 */
#define PLUME_VANLEER_MAX_ITER 100

/* ---- GSPH Riemann-problem states (MINI_DERIVATIVE_COND, options.h:156-170,
 *      559-573): zeroth order (the particles' own states) or linear in the
 *      calc_gradients gradients, with a fallback where a state turns
 *      negative --------------------------------------------------------- */
#define PLUME_RECON_NONE       0   /* linear, no fallback                      */
#define PLUME_RECON_EACH       1   /* per variable and side                    */
#define PLUME_RECON_PAIRWISE   2   /* density / pressure on both sides         */
#define PLUME_RECON_ALL        3   /* every variable on both sides             */
#define PLUME_RECON_ZEROTH     4   /* zeroth order (1D default)                */
#define PLUME_RECON_EACH_SHOCK 10  /* EACH, plus zeroth-order velocities where
                                      3 |u_l - u_r| > min(c_i, c_j) (3D default) */

/* Compile-time switches and physical constants of the reference, as a
 * runtime struct.  Field comments give the reference symbol. */
typedef struct PlumeOptions {
    int    dim;                 /* CODE_DIMENSION: 1 or 3                      */
    int    precision;           /* PLUME_PREC_*                                */
    int    kernel;              /* PLUME_KERNEL_*                              */
    int    lans;                /* HAVE_TURBULENCE_LANS: 0 or 1                */
    int    energy_smooth;       /* HAVE_ENERGY_SMOOTH: 0 or 1 (normalised)     */
    int    pghost_contrib;      /* PGHOST_CONTRIBUTE_DES: 0, 1 or 2            */
    int    adaptive_sml;        /* ADAPTIVE_SML: 0 or 1                        */
    int    sml_interval;        /* SML_UPDATE_INT (3D); 1 = every step (1D)    */
    int    num_loop;            /* num_loop_P                                  */
    double thresh;              /* thresh_P                                    */
    double c_smooth;            /* C_smooth_P                                  */
    double eta_smooth;          /* eta_smooth_P                                */
    double alpha, beta, ata;    /* alf_P, beta_P, ata_P                        */
    double cfl;                 /* CFL_P                                       */
    double cutoff2;             /* CUTOFF2 (12 in 1D, 8 in 3D)                 */
    double list_factor;         /* 4.25, neighs.cc:84                          */
    double g;                   /* g_P                                         */
    double ng0, cvs, cvg, cva, rg, ra; /* ng0_P Cvs_P Cvg_P Cva_P Rg_P Ra_P    */
    double vent_z;              /* Ll_P[2]: erupt ghosts turn real at z>=vent_z */
    double sml_phase2;          /* matprops->smoothing_length                  */
    /* TimeProps (properties.h:17-69); times in seconds, TIME_SCALE = 1 */
    double max_time;
    double timeoutput;
    double stat_erupt, end_erupt;
    int    max_steps;
    int    max_per_bucket;      /* MAX_PARTICLES_PER_BUCKET                    */
    size_t capacity;            /* device particle capacity of the context     */
    int    method;              /* PLUME_METHOD_* (USE_GSPH)                   */
    int    gsph_solver;         /* PLUME_RIEMANN_* (RIEMANN_SOLVER)            */
    int    gsph_recon;          /* PLUME_RECON_* (MINI_DERIVATIVE_COND)        */
    int    gsph_vol;            /* GSPH_SPECIFIC_VOL_APP: 0 interface at the
                                   midpoint, 1 linear, 3 cubic specific volume
                                   (Compute_sij_star, sph_lib.cc:1655-1692)   */
    int    gsph_mono;           /* GSPH_MODIFIED_MONOTONICITY: 0 or 1 (|u_j-u_i|) */
    int    gsph_gradients;      /* 1: calc_gradients every GSPH step, as the
                                   reference does; 0: only when the
                                   reconstruction reads them                  */
    int    gsph_wave_speed;     /* HLL_WAVE_SPEED_EVA of PLUME_RIEMANN_HLLC_MY
                                   (options.h:194-206): 2 Davis, 3 Toro --
                                   the settings the reference runs with (0
                                   stops it, 1, 4 and 5 do not compile);
                                   unused by the other solvers                */
} PlumeOptions;

/* Bucket grid (the background mesh of src/datstr/bucket.h).  Bucket (i,j,k)
 * spans [mindom + i*del, mindom + (i+1)*del) per axis (preprocess.cc:167-177).
 * 1D uses nb[1] = nb[2] = 1 and no bucket rule (every particle is a neighbour
 * candidate, add_air.cc:470-479). */
typedef struct PlumeGrid {
    double mindom[3];
    double del;                 /* bucket edge = PARTICLE_DENSITY * h0         */
    int    nb[3];               /* buckets per axis                            */
    int    subcells;            /* fine cells per bucket edge (GPU tiling)     */
    const uint8_t *flags;       /* nb0*nb1*nb2 PLUME_BUCKET_* (x fastest), may
                                   be NULL (all active, none absorbing/mixed) */
    const int8_t  *face_index;  /* 6 per bucket: bucket_index of bucket.h:
                                   -1/0/1 per face (x-,x+,y-,y+,z-,z+); may be
                                   NULL                                       */
    double domain_lo[3];        /* original domain Ll_P (escape planes)        */
    double domain_hi[3];        /* original domain Lu_P                        */
} PlumeGrid;

/* Structure of arrays on the host.  Pointers for unused axes (1D) may be
 * NULL on upload; on download every non-NULL pointer is filled. */
typedef struct PlumeSoA {
    uint64_t *key;
    double *x, *y, *z;
    double *vx, *vy, *vz;          /* state_vars[1..D]                          */
    double *vsx, *vsy, *vsz;       /* smoothed_v (LANS)                         */
    double *mass, *h;
    double *rho, *e;               /* state_vars[0], state_vars[D+1]            */
    double *p, *Y, *gamma, *c, *T, *cp;
    uint8_t *phase;                /* 1 air, 2 erupted material                 */
    uint8_t *bc_type;              /* PLUME_BC_*                                */
    uint8_t *involved;             /* 0, 1, 2                                   */
} PlumeSoA;

typedef struct PlumeStepLog {
    double dt;                     /* dt of the step after incrtime clipping    */
    double time;                   /* simulated time after the step             */
    int    step;                   /* TimeProps::step after the step            */
    int    status;                 /* PLUME_* of the step                       */
    uint64_t n_total;              /* particles after the step                  */
    uint64_t n_real;               /* need_neigh particles after the step       */
    uint64_t n_lost;               /* particles deleted during the step         */
} PlumeStepLog;

typedef struct plume_ctx plume_ctx;

/* Create a context on the current CUDA device. */
int plume_create(const PlumeOptions *opt, const PlumeGrid *grid, plume_ctx **out);
int plume_destroy(plume_ctx *ctx);

/* Replace all particles (host arrays). */
int plume_upload(plume_ctx *ctx, const PlumeSoA *host, size_t n);
/* Replace all particles from arrays that already live in device memory of
 * the context's device (same layout as PlumeSoA; NULL axes allowed in 1D). */
int plume_upload_device(plume_ctx *ctx, const PlumeSoA *dev, size_t n);
/* Append particles (inlet injection, new ghosts). */
int plume_append(plume_ctx *ctx, const PlumeSoA *host, size_t n);

/* Overwrite the state of ghost particles identified by key: state is n rows
 * of (rho, vx, vy, vz, e) in 3D or (rho, vx, e) in 1D; Y may be NULL.  The
 * equation of state is re-evaluated for them (bcond.cc:214-219). */
int plume_set_ghost_state(plume_ctx *ctx, const uint64_t *keys,
                          const double *state, const double *Y, size_t n);

/* One step in reference order; *dt_out receives the clipped dt. */
int plume_step(plume_ctx *ctx, double *dt_out);
/* nsteps steps without host synchronisation between them; log may be NULL
 * or point to nsteps entries. */
int plume_steps(plume_ctx *ctx, int nsteps, PlumeStepLog *log);

/* One adaptive_sml pass at the current state, with neighbour candidates
 * taken at the current positions (the 1D solver calls adaptive_sml once
 * before its time loop, src/plume/main.cc:643-649). */
int plume_adapt_sml(plume_ctx *ctx);

/* Particle count (total and need_neigh). */
int plume_count(plume_ctx *ctx, size_t *n_total, size_t *n_real);
/* Copy all particles to host arrays of capacity cap; *n receives the count. */
int plume_download(plume_ctx *ctx, PlumeSoA *host, size_t cap, size_t *n);
/* Simulated time, step counter and output counter (TimeProps). */
int plume_get_time(plume_ctx *ctx, double *time, int *step, int *ioutput);
int plume_set_time(plume_ctx *ctx, double time, int step, int ioutput,
                   double next_output);

/* Neighbour pairs (key_i, key_j) for every need_neigh particle i.
 *   mode 0: the candidate list of search_neighs_consth (3D: own bucket plus
 *           particles of the 26 adjacent buckets inside the 4.25 h_i box;
 *           1D: every particle), at the current positions and h;
 *   mode 1: the pairs that the momentum sweep sums over: candidates j != i
 *           inside the CUTOFF2*h_i box whose kernel with h_ij=(h_i+h_j)/2 is
 *           non-zero.
 * If cap is smaller than the pair count nothing is written and *n receives
 * the count. */
int plume_neighbor_pairs(plume_ctx *ctx, int mode, uint64_t *key_i,
                         uint64_t *key_j, size_t cap, size_t *n);

/* plume_neighbor_pairs restricted to the need_neigh particles whose keys are
 * among keys[0..nkeys) (any order): the neighbour vectors of chosen
 * particles, as the reference reads them from one particle of its table
 * (THashTable::lookup(key)->get_neighs(), particle.h:538-541), so large
 * tables can be checked on a sample. */
int plume_neighbor_pairs_of(plume_ctx *ctx, int mode, const uint64_t *keys, size_t nkeys,
                            uint64_t *key_i, uint64_t *key_j, size_t cap, size_t *n);

/* ---- output snapshots ---------------------------------------------------
 * The fields that write_h5part writes (h5part_writer.cc:41-275: x, y, z,
 * vx, vy, vz, rho, e, Y, p, phase, bc_type; plus key, mass and h) of the
 * current particles, staged on the device and copied to the caller's host
 * arrays on a side stream while the caller keeps stepping.
 * plume_snapshot_begin: host needs key, x, vx, rho, e, Y, p, mass, h,
 *   phase, bc_type (and y, z, vy, vz in 3D); involved is filled when not
 *   NULL; other pointers are ignored.  Rows are every particle (ghosts
 *   too, bc_type tells them apart), in the context's order.
 *   Page-locked host arrays are filled by the device directly.  Returns
 *   after the staging is queued; PLUME_E_CAPACITY if cap is too small.
 * plume_snapshot_end: waits for the copy; *n rows, the time and step of the
 *   snapshot.  One snapshot in flight per context. */
int plume_snapshot_begin(plume_ctx *ctx, PlumeSoA *host, size_t cap);
int plume_snapshot_end(plume_ctx *ctx, size_t *n, double *time, int *step);

/* Gradients of the last GSPH step (calc_gradients, calculate_gradient.cc:
 * 22-208: the renormalised SPH gradient of rho, the D velocity components
 * and p of every particle over its neighbour list, zero when the list holds
 * 20 particles or fewer inside the CUTOFF2*h box), with the keys of their
 * rows.  grad receives (D+2)*D doubles per particle: d rho/dx_k, d v_0/dx_k,
 * ..., d p/dx_k (k fastest).  PLUME_E_INVALID when the last step computed
 * none (method SPH, or zeroth-order reconstruction with gsph_gradients 0).
 * If cap is smaller than the particle count nothing is written and *n
 * receives the count. */
int plume_gsph_gradients(plume_ctx *ctx, uint64_t *key, double *grad, size_t cap, size_t *n);

/* ---- domain growth (ADJUST_DOMAIN, main.cc:257-300, 433-436) ----------
 * Every bucket carries an involvement state (PLUME_BINV_*), initially NONE
 * for PLUME_BUCKET_ABSORBING buckets and POTENTIAL for the others
 * (dataread.cc:457); plume_set_bucket_involvement overrides it (e.g. BOTH
 * for the vent buckets, setup_influx.cc:206-209).
 *
 * plume_scan_outside_layer (scan_outside_layer.cc:37-121, run by the
 * reference after every 3D step): a POTENTIAL bucket holding an involved
 * particle (involved == 2) becomes BOTH; *adapt receives how many of those
 * border a non-empty NONE bucket that is not UNDERGROUND (the reference's
 * trigger for adapt_domain).
 * plume_adapt_domain (adapt_domain.cc:41-194): every non-empty NONE bucket
 * that is neither UNDERGROUND nor PRESS_BC and borders a bucket with
 * involved particles (state bit 1) becomes POTENTIAL and stops absorbing;
 * its particles turn real (bc 100) and potentially involved (1): on-ground
 * MIXED buckets their pressure ghosts, other MIXED buckets those inside the
 * domain (Bucket::determine_escape, bucket.cc:435-452), OVERGROUND buckets
 * all.  The new pressure-ghost and wall-ghost layers of the reference's
 * add_pressure_ghost / add_wall_ghost are particle creation on the host
 * (plume_append), with a new image table (plume_set_wall_images). */
int plume_set_bucket_involvement(plume_ctx *ctx, const uint8_t *state, size_t nbuckets);
int plume_get_bucket_involvement(plume_ctx *ctx, uint8_t *state, size_t nbuckets);
int plume_scan_outside_layer(plume_ctx *ctx, int *adapt);
int plume_adapt_domain(plume_ctx *ctx);

/* The hydrostatic atmosphere of ATMOSPHERE_TYPE 1 (air_prop_hydro,
 * sph_lib.cc:488-592; constants of parameters.h:902-935). */
typedef struct PlumeAtmosphere {
    double Ta0, pa0, Ra, gamma;           /* Ta0_P pa0_P Ra_P gamma_P          */
    double H1, H2, H3, miu1, miu2;        /* layer heights and lapse rates      */
    double Ata1, Ate1, Ata2, Atb2, Ata3, Atb3, AtC3, Ate3; /* pressure fit     */
} PlumeAtmosphere;

/* The pressure-ghost layers that follow an adaptation (add_pressure_ghost,
 * add_pressure_ghost.cc:37-316; main.cc:265-271), on the device: every NONE
 * bucket that holds no pressure ghost and has a neighbour whose state is not
 * NONE is made active and filled with a lattice of spacing
 * sml_phase2 (edge / spacing points per axis, at corner + spacing/2 + i
 * spacing; on-ground MIXED buckets above the ground only; UNDERGROUND
 * buckets none) of pressure ghosts at rest in the hydrostatic air of their
 * height (initial_air, sph_lib.cc:831-866: mass of the particle's box by the
 * reference's three-point rule, then the mixture EOS).  The new rows get
 * keys key_base, key_base + 1, ... (bucket by bucket, x fastest, then the
 * lattice with z fastest); *added is their number.  Single-run 3D
 * contexts; PLUME_E_CAPACITY when the table would overflow. */
int plume_add_pressure_ghost(plume_ctx *ctx, const PlumeAtmosphere *atm, uint64_t key_base,
                             size_t *added);

/* The wall-ghost layers of a grown domain (add_wall_ghost,
 * add_wall_ghost.cc:44-293; main.cc:279), on the device: every on-ground
 * MIXED bucket (bottom face below the ground) that holds particles but no
 * wall ghost gets wall ghosts (bc 2) on its lattice points below the ground
 * plane, and the bucket below it is made active and filled whole; lattice,
 * state, keys and errors as plume_add_pressure_ghost. */
int plume_add_wall_ghost(plume_ctx *ctx, const PlumeAtmosphere *atm, uint64_t key_base, size_t *added);

/* The air of add_air (add_air.cc:490-795, 3D), on the device: every empty
 * bucket whose involvement state is not NONE is made active; MIXED and
 * OVERGROUND ones are filled with real air particles (bc 100, potentially
 * involved) on the lattice of plume_add_pressure_ghost (on-ground MIXED:
 * above the ground only), PRESS_BC and UNDERGROUND ones stay empty.  State,
 * keys and errors as plume_add_pressure_ghost. */
int plume_add_air(plume_ctx *ctx, const PlumeAtmosphere *atm, uint64_t key_base, size_t *added);

/* The adaptation block of the 3D loop (main.cc:257-295) in one call:
 * plume_scan_outside_layer; when it asks for it (*adapted != 0),
 * plume_adapt_domain, plume_add_pressure_ghost, plume_add_wall_ghost (keys
 * from key_base on, *added in all) and, when wall images are in use,
 * plume_search_bnd_images and plume_apply_bcond.  (move_data,
 * shift_brief_buck and update_bgmesh have nothing to do in a one-GPU
 * table.) */
int plume_adapt_step(plume_ctx *ctx, const PlumeAtmosphere *atm, uint64_t key_base, int *adapted,
                     size_t *added);

/* Per-phase device time of the last plume_step/plume_steps call, summed over
 * its steps, in ms (CUDA events on the context's stream):
 * [0] search (keys, sort, gather, cell table), [1] adaptive h, [2] bucket
 * max h and per-step neighbour lists, [3] momentum/energy sweep, [4] its commit + EOS, [5] density sweep,
 * [6] its commit + EOS, [7] velocity filter, [8] position update and
 * re-bucketing, [9] dt reduction, [10] total, [11] the momentum pair-sweep
 * kernel alone (inside [3]), [12] eruption inlet (add_new_erupt) and the
 * step's end, [13] wall boundary (apply_bcond).  n <= 14 entries. */
int plume_phase_times(plume_ctx *ctx, float *ms, int n);

/* Device kernel launches issued by the last plume_step/plume_steps call. */
int plume_launch_count(plume_ctx *ctx, uint64_t *n);

/* Text of the last error of ctx (or of the last failed create if ctx is
 * NULL). */
int plume_last_error(plume_ctx *ctx, char *buf, size_t len);

/* ---------------------------------------------------------------- ensembles
 * An ensemble context holds nmembers independent runs (members) in one
 * particle table: every particle carries its member id; each member has its
 * own bucket grid, time state (dt, time, step, output counter) and the
 * per-member options (cfl, ng0, cvs, cvg, cva, rg, ra, vent_z, sml_phase2,
 * max_time, timeoutput, stat_erupt, end_erupt, max_steps).  All other
 * options must be equal across members.  Every kernel of a step covers the
 * particles of all members in one launch; a member never sees another
 * member's particles and computes what it would compute alone (bit for bit
 * in FP64).  A member stops stepping at its own TimeProps::ifend
 * (properties.h:76-79), or at its first error status (where the reference
 * asserts and aborts the run), while the others go on: the ensemble entry
 * points do not return members' statuses, plume_batch_time does.  No
 * counterpart in the
 * reference, which runs one problem per process: this is the batched path
 * for parameter sweeps and ensembles.
 *
 * plume_batch_create: options[m] and grids[m] for m < nmembers; the
 *   context's capacity is the sum of options[m].capacity.  The single-run
 *   entry points (plume_step, plume_steps, plume_count, plume_download,
 *   plume_neighbor_pairs, plume_set_ghost_state ...) work on ensembles too;
 *   plume_get_time reports member 0 and plume_set_time sets every member.
 * plume_batch_upload / plume_batch_append: particles of any members, member
 *   ids per row (< nmembers).
 * plume_batch_download: plume_download plus the member id of every row.
 * plume_batch_time: per-member time, step, running flag (0 once the member
 *   reached its end or failed) and status (PLUME_OK or the PLUME_E_* code
 *   that stopped it); arrays of nmembers entries, any may be NULL.
 * plume_batch_run: steps every running member until all have ended or
 *   max_steps steps were issued.  graph_steps > 0 captures that many steps
 *   into one CUDA graph and replays it (the host checks the members between
 *   replays; ended members idle inside a replay); 0 issues steps one by
 *   one.  Members of a single-run context are stopped at their end as well.
 *   plume_phase_times reports the run's device time in [10]. */
#define PLUME_MAX_MEMBERS 65535
int plume_batch_create(const PlumeOptions *options, const PlumeGrid *grids, int nmembers,
                       plume_ctx **out);
int plume_batch_upload(plume_ctx *ctx, const PlumeSoA *host, const uint16_t *member, size_t n);
int plume_batch_append(plume_ctx *ctx, const PlumeSoA *host, const uint16_t *member, size_t n);
int plume_batch_download(plume_ctx *ctx, PlumeSoA *host, uint16_t *member, size_t cap, size_t *n);
int plume_batch_time(plume_ctx *ctx, double *time, int *step, int *running, int *status);
int plume_batch_run(plume_ctx *ctx, int max_steps, int graph_steps, int *steps_done);

/* ---------------------------------------------------------------- wall boundary
 * The wall-ghost states of apply_bcond (src/plume/bcond.cc:24-249, the
 * reference's BC_FOR_KX 1), on the device.  plume_set_wall_images sets the
 * image table that search_bnd_images (datstr/bnd_image.cc:35-245) builds:
 * for each wall ghost (bc_type 2, key ghost_keys[i]) its image point
 * image_xyz[3i..3i+2]; n = 0 clears it.  Every step then starts, after its
 * sort, by setting each such ghost's rho, v, e, Y to the normalised SPH
 * averages of the real and pressure-ghost particles around its image (the
 * image's bucket and its 26 neighbours), the velocity reflected in the wall,
 * and its EOS fields -- where the reference applies the same at the end of
 * the previous step and once before its loop.  plume_apply_bcond applies it
 * now (a host that downloads after plume_steps and wants the states the
 * reference writes at the end of the last step).  3D, keys unique in the
 * context; the adjoint entry points reject a context with images. */
int plume_set_wall_images(plume_ctx *ctx, const uint64_t *ghost_keys, const double *image_xyz, size_t n);

/* The image table of search_bnd_images (bnd_image.cc:36-245) for a flat
 * ground, found on the device from the current particles and installed as
 * plume_set_wall_images would: every wall ghost (bc 2) of a MIXED bucket
 * whose own bucket or a neighbour is an on-ground MIXED bucket (bottom face
 * below the ground plane, top face not) gets the image (x, y, 2 z_ground -
 * z).  *n = the number of images.  Single-run 3D contexts.  Call it after
 * the wall ghosts change (plume_add_wall_ghost, plume_append). */
int plume_search_bnd_images(plume_ctx *ctx, size_t *n);
int plume_apply_bcond(plume_ctx *ctx);

/* ---------------------------------------------------------------- eruption inlet
 * add_new_erupt (src/plume/setup_erupt.cc:389-673) on the device.  While
 * TimeProps::iferupt, every step ends by adding, for each duct column, the
 * particles the inflow has made room for since the previous step:
 * n = floor((fmod(t - dt, t_each) + dt) / t_each), t_each = spacing / vel,
 * at z = bot + (t_add + i t_each) vel, with the vent state (Particle
 * constructor, datstr/particle.cc:210-316: v = (0, 0, vel), Y, phase 2,
 * bc_type 0, T and cp from the EOS, p, c and gamma the given values).  The
 * key of a column's k-th particle is key_base + k ncol + column (col_count:
 * particles already added per column, NULL = 0).  New particles take rows
 * after the live ones; reserve_per_step bounds how many one step adds
 * (more: PLUME_E_CAPACITY), and every step's sort covers that many extra
 * rows.  NULL or ncol = 0 clears the inlet.  One 3D run; the adjoint entry
 * points reject a context with an inlet. */
typedef struct PlumeInlet {
    size_t ncol;
    const double *col_xy;               /* 2 per column                         */
    const double *col_vel;              /* inflow velocity per column (> 0)      */
    const unsigned long long *col_count;
    double bot;                         /* simprops bot: duct bottom             */
    double spacing;                     /* sml_of_phase2: particle spacing       */
    double mass, h;                     /* mass_of_phase2, RATIO_SML_DX * spacing */
    double rho, e, p, gamma, c, Y;      /* rhov_P, ev0_P, pv0_P, gamma_v_P, 340, 1 */
    uint64_t key_base;
} PlumeInlet;
int plume_set_inlet(plume_ctx *ctx, const PlumeInlet *inlet, int reserve_per_step);

/* ---------------------------------------------------------------- adjoint
 * Reverse-mode derivatives of a window of particle steps (one 3D run, FP64,
 * Gaussian kernel).  No counterpart in the reference.
 *
 * plume_adjoint_record: runs nsteps steps like plume_steps and keeps the
 *   state every checkpoint_every steps (and at the end).
 * plume_adjoint_backward: given the adjoint of a scalar objective J with
 *   respect to the window's final state (final_bar: rows matched by key to
 *   the particles alive at the end; PlumeSoA fields x .. cp, gamma ignored,
 *   NULL arrays = zero), returns dJ/d(first state) in initial_bar (rows in
 *   the order of the window's first state, keys filled; cap >= its row
 *   count, returned in n_initial) and dJ/d ng0 (the mixture constant of the
 *   EOS).  Each checkpoint segment is recomputed with per-step snapshots and
 *   differentiated stage by stage (position, LANS filter, density + EOS,
 *   momentum/energy, adaptive h, dt).  The discrete decisions of the
 *   recorded run are kept: neighbour lists, the particle that sets dt,
 *   erupt-to-real conversions, deletions; a dt clipped to an output or end
 *   time inside the window is rejected (PLUME_E_INVALID).  After the call
 *   the context holds the window's final state again. */
int plume_adjoint_record(plume_ctx *ctx, int nsteps, int checkpoint_every);
int plume_adjoint_backward(plume_ctx *ctx, const PlumeSoA *final_bar, size_t n_final,
                           PlumeSoA *initial_bar, size_t cap, size_t *n_initial, double *ng0_bar);

/* Time step without allocating: dt_out[0] = cfl * min(h[i] / c[i]) over the
 * particles with bc_type 100 or 99 (1.0e10 when there are none), from
 * device arrays of n particles, on `stream` (a cudaStream_t; NULL = the
 * default stream).  No counterpart in the reference: it is the dt reduction
 * of plume_step offered to callers that cannot allocate GPU memory (hosts
 * whose device memory belongs to their own pool, code paths where an
 * allocation would synchronise the device).  Its scratch is a fixed device
 * array of PLUME_NOALLOC_MAX_BLOCKS doubles that every GPU loading the
 * library keeps until exit; n above PLUME_NOALLOC_MAX_BLOCKS *
 * PLUME_NOALLOC_CHUNK returns PLUME_E_CAPACITY.  The first call on a device
 * looks up that array's address (again after the device's context is
 * replaced, e.g. by cudaDeviceReset); make it before any stream capture.
 * Calls share the array: calls that overlap on the GPU race.  A particle
 * with h <= 0 or c <= 0 (or NaN) among those particles gives a NaN dt.
 * Asynchronous: read dt_out after synchronising the stream. */
#define PLUME_NOALLOC_MAX_BLOCKS 1024
#define PLUME_NOALLOC_CHUNK      16384
int plume_timestep_noalloc(const double *h, const double *c, const uint8_t *bc_type,
                           size_t n, double cfl, double *dt_out, void *stream);

/* ---- bucket grid ------------------------------------------------------
 * The preprocessor's bucket grid for a flat-ground domain (preprocess.cc:
 * 68-177, 386-464; the funkyNNNN.h5 files that Read_Grid loads,
 * dataread.cc:247), computed on the device: the original domain [lo, hi]
 * padded by 1.5 buckets of edge 8 * h0, bucket counts rounded up, and the
 * face indices and types of every bucket (MIXED; absorbing with
 * PLUME_BUCKET_UNDERGROUND or PLUME_BUCKET_PRESS_BC; OVERGROUND none).
 * Fills grid (mindom, del, nb, subcells, domain_lo/hi) and *nbk (buckets,
 * x fastest); with flags and face_index (host arrays of cap and 6 * cap
 * entries) also those, and points grid->flags / face_index at them.  Call
 * with flags NULL to size.  PLUME_E_CAPACITY when *nbk > cap. */
int plume_grid_generate(const double lo[3], const double hi[3], double h0, int subcells,
                        PlumeGrid *grid, uint8_t *flags, int8_t *face_index, size_t cap,
                        size_t *nbk);

/* ---- the initial vent duct --------------------------------------------
 * setup_erupt (setup_erupt.cc:44-388; main.cc:156), on the device: the
 * erupt ghosts of the duct below the vent -- the box [-radius, radius]^2 x
 * [z_top - depth, z_top] filled with np particles' worth of lattice
 * (Compute_mass, sph_lib.cc:1024-1040: spacing = cbrt(volume / np), mass =
 * rho volume / np), points stepped out from the vent axis, kept where
 * x^2 + y^2 <= radius^2 -- with the state of the erupt-ghost constructor
 * (particle.cc:210-316: rho, e, vertical speed of the profile
 * (ERUPT_VELOCITY_PROF 0 uniform u_avg, 1 parabolic 2 u_avg (1 - r^2/R^2)),
 * Y 1, phase 2, the mixture EOS, then p, c and gamma as given); the
 * particles other than erupt ghosts inside the duct are removed.  Keys
 * key_base, key_base + 1, ... (z layer by layer from the top, then the
 * points in the reference's order); *mass and *sml (may be NULL) return the
 * duct particles' mass and spacing (simprops mass_of_phase2 /
 * sml_of_phase2, which the eruption inlet uses). */
typedef struct PlumeDuct {
    double x0, y0;              /* vent axis (Pos_v_P)                        */
    double z_top, depth;        /* Ll_P[2]; EXT_DOM_COF*PARTICLE_DENSITY*h0   */
    double radius;              /* rv_P                                       */
    int    np;                  /* num_erupt_particles                        */
    int    profile;             /* ERUPT_VELOCITY_PROF: 0 uniform, 1 parabolic */
    double u_avg;               /* Vv0_P                                      */
    double rho, e, p, gamma, c; /* rhov_P ev0_P pv0_P gamma_v_P sndspd        */
} PlumeDuct;
int plume_setup_erupt(plume_ctx *ctx, const PlumeDuct *duct, uint64_t key_base, size_t *added,
                      size_t *removed, double *mass, double *sml);

/* Library version string "major.minor.patch". */
const char *plume_version(void);

#ifdef __cplusplus
}
#endif
#endif /* PLUME_GPU_H */
