/*
 * sph_oracle.h -- CPU oracle of the Plume-SPH particle step.
 *
 * TEST INFRASTRUCTURE.  This is the checker, not the product: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm may
 * load it.  It restates, in plain C over structure-of-arrays particles, the
 * per-step algorithm of the reference solver (file:line citations in
 * sph_oracle.c) with the reference's operation order, so that it agrees with
 * the reference build (oracle/_ref, see oracle/Makefile) to the last bit on
 * the first step and to rounding afterwards.
 *
 * Parity pin: tests/test_oracle_golden.py checks this oracle against golden
 * vectors produced by running the reference's own source files
 * (tests/golden/make_golden.py).
 */
#ifndef SPH_ORACLE_H
#define SPH_ORACLE_H

#include <stddef.h>
#include <stdint.h>
#include "../include/plume_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* TimeProps (src/datstr/properties.h:17-69) with TIME_SCALE = 1. */
typedef struct OracleTime {
    double time;          /* current time                                   */
    double dtime;         /* dt of the last step                            */
    double ndtimeoutput;  /* next output time                               */
    int    step;
    int    ioutput;
} OracleTime;

/* One adaptive_sml pass (neighs.cc:479-693) with the current lists. */
int oracle_adaptive(const PlumeOptions *opt, const PlumeGrid *grid,
                    PlumeSoA *s, size_t n, int nthreads);

/* nsteps steps of the hot loop.  *n is updated when particles are deleted
 * (arrays are compacted in order).  dt_log (may be NULL) receives the
 * clipped dt of each step.  Returns PLUME_OK or a PLUME_E_* code. */
/* Wall boundary (apply_bcond, bcond.cc:24-249): every image (ghost key,
 * image point) sets its wall ghost's state.  oracle_steps_bc applies it at
 * the end of every 3D step (main.cc:468). */
int oracle_apply_bcond(const PlumeOptions *opt, const PlumeGrid *grid, PlumeSoA *s, size_t n,
                       const uint64_t *img_key, const double *img_xyz, size_t nimg);
int oracle_steps_bc(const PlumeOptions *opt, const PlumeGrid *grid, PlumeSoA *s, size_t *n,
                    OracleTime *t, int nsteps, double *dt_log, int nthreads,
                    const uint64_t *img_key, const double *img_xyz, size_t nimg);
/* oracle_steps_bc plus the eruption inlet (add_new_erupt,
 * setup_erupt.cc:389-673) after the re-bucketing of every 3D step; the
 * particle arrays hold cap rows; par = bot, spacing, mass, h, rho, e, p,
 * gamma, c, Y of the vent; col_count is updated. */
int oracle_steps_inlet(const PlumeOptions *opt, const PlumeGrid *grid, PlumeSoA *s,
                       size_t *n, size_t cap, OracleTime *t, int nsteps, double *dt_log,
                       int nthreads, const uint64_t *img_key, const double *img_xyz,
                       size_t nimg, const double *col_xy, const double *col_vel,
                       uint64_t *col_count, size_t ncol, const double *par,
                       uint64_t key_base);
int oracle_steps(const PlumeOptions *opt, const PlumeGrid *grid,
                 PlumeSoA *s, size_t *n, OracleTime *t, int nsteps,
                 double *dt_log, int nthreads);
/* oracle_steps plus the GSPH gradients of the last step (calc_gradients,
 * calculate_gradient.cc:22-208): (D+2)*D doubles per row, rows with their
 * keys; *n_grad = 0 when the step computed none. */
int oracle_steps_grad(const PlumeOptions *opt, const PlumeGrid *grid, PlumeSoA *s,
                      size_t *n, OracleTime *t, int nsteps, double *dt_log, int nthreads,
                      double *grad, uint64_t *grad_key, size_t cap, size_t *n_grad);

/* Domain growth (3D): scan_outside_layer and adapt_domain, the semantics
 * of plume_scan_outside_layer / plume_adapt_domain; binv: per-bucket
 * involvement states (in/out); flags (may be NULL): the bucket flags, whose
 * ABSORBING bit adapt_domain clears on the buckets it converts. */
int oracle_scan_outside_layer(const PlumeOptions *opt, const PlumeGrid *grid, const PlumeSoA *s, size_t n,
                              uint8_t *binv, int *adapt);
int oracle_adapt_domain(const PlumeOptions *opt, const PlumeGrid *grid, PlumeSoA *s, size_t n,
                        uint8_t *binv, uint8_t *flags);

/* Neighbour pairs, same modes as plume_neighbor_pairs(). */
int oracle_pairs(const PlumeOptions *opt, const PlumeGrid *grid,
                 const PlumeSoA *s, size_t n, int mode,
                 uint64_t *key_i, uint64_t *key_j, size_t cap, size_t *npairs);
int oracle_pairs_of(const PlumeOptions *opt, const PlumeGrid *grid,
                    const PlumeSoA *s, size_t n, int mode,
                    const uint64_t *keys, size_t nkeys,
                    uint64_t *key_i, uint64_t *key_j, size_t cap, size_t *npairs);

/* Bounded CPU sample of one step: the neighbour search and the pair sweeps
 * of a step run for the first `ntarget` need_neigh particles only (all
 * other work of the step is per-particle streaming and is included for all
 * particles).  Returns the wall seconds, or a negative value on error.
 * The particle state is not modified. */
double oracle_sample_step_seconds(const PlumeOptions *opt,
                                  const PlumeGrid *grid, const PlumeSoA *s,
                                  size_t n, size_t ntarget, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
