/*
 * sph_oracle.c -- CPU oracle of the Plume-SPH per-step particle path.
 *
 * TEST INFRASTRUCTURE (the checker, never the product).  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm load
 * it.  It restates the reference algorithm over structure-of-arrays
 * particles; every function cites the reference lines it follows (paths
 * inside the Plume-SPH source tree).  Operation order inside each formula is
 * kept as the reference writes it, so that with the same libm the first
 * step agrees with the reference build to the last bit.  Build with
 * -ffp-contract=off (x86 compilers do not fuse by default; aarch64 ones do).
 *
 * Parity pin: golden vectors from the reference's own sources
 * (tests/golden/make_golden.py, tests/test_oracle_golden.py).
 */
#include "sph_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* constants of src/plume/constant.h and sph_lib.cc */
#define OR_T1        0.564189583547756   /* 1/sqrt(pi), sph_lib.cc:206     */
#define OR_CUTOFF    3.0                 /* CUTOFF, constant.h:51          */
#define OR_EPS_HALF  0.4                 /* EPSILON_HALF, constant.h:94    */
#define OR_PRANDTL   0.85                /* PRANDTL_NUM, constant.h:95     */
#define OR_E_SMOOTH  4.0                 /* E_SMOOTH_RATIO, constant.h:185 */
#define OR_MSFRC_TH  1.0e-6              /* MSFRC_THRESH, constant.h:80    */
#define OR_TINY      1.0e-8              /* TINY, constant.h:76            */
#define OR_C_SHOCK   3.0                 /* C_SHOCK, constant.h:103        */
/* cubic B-spline normalisations (1D: 2/3, 3D: 1/pi) */
#define OR_M4_S1     0.66666666666666663
#define OR_M4_S3     0.31830988618379069

/* ------------------------------------------------------------------ */
/* particle predicates, src/datstr/particle.h:555-615                   */
/* ------------------------------------------------------------------ */
static inline int need_neigh(uint8_t bc) { return bc == 100 || bc == 99; }
static inline int is_real(uint8_t bc) { return bc == 100 || bc == 99; }
static inline int contr_dens(uint8_t bc, int mode)
{
    /* particle.h:570-579 (PGHOST_CONTRIBUTE_DES) */
    if (mode == 1) return bc == 100 || bc == 99 || bc == 1;
    if (mode == 2) return bc == 100 || bc == 99 || bc == 1 || bc == 0;
    return bc == 100 || bc == 99;
}
static inline int contr_vel_smooth(uint8_t bc)
{
    return bc == 100 || bc == 99 || bc == 2; /* particle.h:587-590 */
}

/* in_support, sph_header.h:49-60: every |dx_k| <= h */
static inline int in_support(const double *dx, double h, int D)
{
    for (int i = 0; i < D; i++)
        if (fabs(dx[i]) > h) return 0;
    return 1;
}

/* ------------------------------------------------------------------ */
/* kernels                                                              */
/* ------------------------------------------------------------------ */
/* weight, sph_lib.cc:210-230 */
static double weight_gauss(const double *s, double h, int D)
{
    for (int i = 0; i < D; i++)
        if (fabs(s[i]) > OR_CUTOFF) return 0;
    double norm = 1, expt = 0;
    for (int i = 0; i < D; i++) {
        norm *= OR_T1 / h;
        expt += s[i] * s[i];
    }
    return norm * exp(-expt);
}
/* d_weight, sph_lib.cc:240-253 */
static double d_weight_gauss(const double *s, double h, int dir, int D)
{
    for (int i = 0; i < D; i++)
        if (fabs(s[i]) > OR_CUTOFF) return 0;
    double tmp = -2 * s[dir] / h;
    return tmp * weight_gauss(s, h, D);
}
/* cubic B-spline with radial support 2h (the Sod / ensemble workloads) */
static double weight_m4(const double *s, double h, int D)
{
    double r2 = 0;
    for (int i = 0; i < D; i++) r2 += s[i] * s[i];
    double q = sqrt(r2);
    if (q >= 2.0) return 0;
    double norm = (D == 1) ? OR_M4_S1 : OR_M4_S3;
    for (int i = 0; i < D; i++) norm = norm / h;
    double w;
    if (q < 1.0) {
        w = 1.0 - 1.5 * q * q + 0.75 * q * q * q;
    } else {
        double t = 2.0 - q;
        w = 0.25 * t * t * t;
    }
    return norm * w;
}
static double d_weight_m4(const double *s, double h, int dir, int D)
{
    double r2 = 0;
    for (int i = 0; i < D; i++) r2 += s[i] * s[i];
    double q = sqrt(r2);
    if (q >= 2.0 || q == 0.0) return 0;
    double norm = (D == 1) ? OR_M4_S1 : OR_M4_S3;
    for (int i = 0; i < D; i++) norm = norm / h;
    double dw;
    if (q < 1.0) {
        dw = -3.0 * q + 2.25 * q * q;
    } else {
        double t = 2.0 - q;
        dw = -0.75 * t * t;
    }
    return norm * dw * s[dir] / (q * h);
}
static inline double kw(int kernel, const double *s, double h, int D)
{
    return kernel == PLUME_KERNEL_M4 ? weight_m4(s, h, D) : weight_gauss(s, h, D);
}
static inline double kdw(int kernel, const double *s, double h, int dir, int D)
{
    return kernel == PLUME_KERNEL_M4 ? d_weight_m4(s, h, dir, D)
                                     : d_weight_gauss(s, h, dir, D);
}

/* compute_F, sph_lib.cc:257-281 */
static double compute_F(const double *dwdx, const double *dx, int D)
{
    double r_sq = 0., W_r = 0.;
    for (int i = 0; i < D; i++) W_r += dwdx[i] * dx[i];
    if (W_r == 0) return 0.0;
    for (int i = 0; i < D; i++) r_sq += dx[i] * dx[i];
    return W_r / r_sq;
}
/* art_vis, sph_lib.cc:402-424 */
static double art_vis(const PlumeOptions *o, double rhoab, double sndspdab,
                      const double *rab, const double *vab, double rsqab,
                      double h, int D)
{
    double vrab = 0., vis = 0.;
    for (int k = 0; k < D; k++) vrab += rab[k] * vab[k];
    double miuab = h * vrab / (rsqab + o->ata * h * h);
    if (vrab > 0)
        vis = 0.;
    else if (vrab < 0)
        vis = (o->beta * miuab - o->alpha * sndspdab) * miuab / rhoab;
    return vis;
}
/* SPH_epsilon_mom, sph_lib.cc:1331-1338 */
static double eps_mom(const double *vab, double Vb, int D)
{
    double dotv = 0.;
    for (int i = 0; i < D; i++) dotv += vab[i] * vab[i];
    return OR_EPS_HALF * dotv * Vb;
}
/* SPH_epsilon_heat_conductivity (6-argument form), sph_lib.cc:1399-1440 */
static double eps_heat(double cp_ab, const double *ds, const double *vab,
                       double hab, double cab, int D)
{
    double dotvv = 0., dotvr = 0., dotrr = 0., kab;
    for (int i = 0; i < D; i++) dotvr += fabs(vab[i] * ds[i]);
    if (dotvr == 0.) return 0.;
    for (int i = 0; i < D; i++) dotrr += ds[i] * ds[i];
    for (int i = 0; i < D; i++) dotvv += vab[i] * vab[i];
    if (D == 3)
        kab = 10.0 * OR_EPS_HALF * cp_ab * dotrr * dotvv / (OR_PRANDTL * dotvr);
    else if (D == 2)
        kab = 8.0 * OR_EPS_HALF * cp_ab * dotrr * dotvv / (OR_PRANDTL * dotvr);
    else
        kab = 0.0;
    return kab / (hab * cab);
}

/* Particle::update_second_var, src/datstr/particle.cc:528-604 (ideal gas) */
static void eos(const PlumeOptions *o, PlumeSoA *s, size_t i)
{
    double desm = s->rho[i];
    double Y = s->Y[i];
    double na = 1 - Y;
    double engr = s->e[i];
    double ng = o->ng0 * Y;
    double ns = Y - ng;
    double Cvm = ns * o->cvs + ng * o->cvg + na * o->cva;
    double Rm = ng * o->rg + na * o->ra;
    double Rmg = Rm / (ng + na);
    double gamma = 1 + Rm / Cvm;
    double desmg = desm * (na + ng);
    double pressure = Rmg * desmg * engr / Cvm;
    s->gamma[i] = gamma;
    s->p[i] = pressure;
    s->c[i] = pow(gamma * pressure / desmg, 0.5);
    s->T[i] = engr / Cvm;
    if (o->lans) s->cp[i] = Cvm;
}

/* ------------------------------------------------------------------ */
/* bucket grid (preprocess.cc:167-177, bucket.h:238-245)                */
/* ------------------------------------------------------------------ */
static int bucket_axis(double x, double mind, double del, int nb)
{
    double f = floor((x - mind) / del);
    if (!(f > -2.0) || !(f < (double)nb + 1.0)) return -1;
    int b = (int)f;
    if (b < 0) b = 0;
    if (b > nb - 1) b = nb - 1;
    while (b > 0 && x < mind + b * del) b--;
    while (b < nb - 1 && x >= mind + (b + 1) * del) b++;
    if (x < mind + b * del || x >= mind + (b + 1) * del) return -1;
    return b;
}
static long bucket_of(const PlumeGrid *g, double x, double y, double z)
{
    int bx = bucket_axis(x, g->mindom[0], g->del, g->nb[0]);
    int by = bucket_axis(y, g->mindom[1], g->del, g->nb[1]);
    int bz = bucket_axis(z, g->mindom[2], g->del, g->nb[2]);
    if (bx < 0 || by < 0 || bz < 0) return -1;
    return ((long)bz * g->nb[1] + by) * g->nb[0] + bx;
}
static uint8_t bucket_flags(const PlumeGrid *g, long b)
{
    return g->flags ? g->flags[b] : 0;
}

/* ------------------------------------------------------------------ */
/* neighbour lists, search_neighs_consth (neighs.cc:37-211)             */
/* ------------------------------------------------------------------ */
typedef struct Lists {
    size_t  *start;   /* n+1 */
    int32_t *idx;
    size_t   nidx;
} Lists;

static void lists_free(Lists *L)
{
    free(L->start);
    free(L->idx);
    memset(L, 0, sizeof(*L));
}

/* Builds, for each of the first `ntarget` need_neigh particles (all of them
 * when ntarget == (size_t)-1), the list: every particle of its own bucket
 * (neighs.cc:89-92), then, for the 26 adjacent buckets in x-major order
 * (preprocess.cc:287-313), the particles inside the list_factor*h_i box
 * (neighs.cc:84,117-131).  Particles of one bucket keep index order. */
static int build_lists_3d_for(const PlumeOptions *o, const PlumeGrid *g,
                              const PlumeSoA *s, size_t n, size_t ntarget,
                              Lists *L, int nthreads, int all, const char *tmask);
static int build_lists_3d(const PlumeOptions *o, const PlumeGrid *g,
                          const PlumeSoA *s, size_t n, size_t ntarget,
                          Lists *L, int nthreads)
{
    return build_lists_3d_for(o, g, s, n, ntarget, L, nthreads, 0, NULL);
}

/* all: lists for every particle, as search_neighs_consth builds them under
 * USE_GSPH (neighs.cc:76, 136: ghosts need lists for their gradients);
 * tmask (when not NULL): lists only for the targets it marks */
static int build_lists_3d_for(const PlumeOptions *o, const PlumeGrid *g,
                              const PlumeSoA *s, size_t n, size_t ntarget,
                              Lists *L, int nthreads, int all, const char *tmask)
{
    long nbk = (long)g->nb[0] * g->nb[1] * g->nb[2];
    long *bk = (long *)malloc(sizeof(long) * (n ? n : 1));
    size_t *bstart = (size_t *)calloc((size_t)nbk + 1, sizeof(size_t));
    int32_t *bidx = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    if (!bk || !bstart || !bidx) { free(bk); free(bstart); free(bidx); return PLUME_E_INVALID; }
    for (size_t i = 0; i < n; i++) {
        bk[i] = bucket_of(g, s->x[i], s->y[i], s->z[i]);
        if (bk[i] < 0) { free(bk); free(bstart); free(bidx); return PLUME_E_OUTSIDE_GRID; }
        bstart[bk[i] + 1]++;
    }
    for (long b = 0; b < nbk; b++) bstart[b + 1] += bstart[b];
    {
        size_t *fill = (size_t *)malloc(sizeof(size_t) * (size_t)(nbk ? nbk : 1));
        memcpy(fill, bstart, sizeof(size_t) * (size_t)nbk);
        for (size_t i = 0; i < n; i++) bidx[fill[bk[i]]++] = (int32_t)i;
        free(fill);
    }
    /* targets */
    size_t nt = 0;
    for (size_t i = 0; i < n; i++)
        if ((all || need_neigh(s->bc_type[i])) && nt < ntarget) nt++;
    L->start = (size_t *)calloc(n + 1, sizeof(size_t));
    size_t *cnt = (size_t *)calloc(n + 1, sizeof(size_t));
    char *is_t = (char *)calloc(n ? n : 1, 1);
    {
        size_t c = 0;
        for (size_t i = 0; i < n && c < nt; i++)
            if (all || need_neigh(s->bc_type[i])) { is_t[i] = 1; c++; }
        if (tmask)
            for (size_t i = 0; i < n; i++) is_t[i] = is_t[i] && tmask[i];
    }
    int nbx = g->nb[0], nby = g->nb[1], nbz = g->nb[2];
    /* two passes: count, then fill */
    for (int pass = 0; pass < 2; pass++) {
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
        for (long ii = 0; ii < (long)n; ii++) {
            size_t i = (size_t)ii;
            if (!is_t[i]) continue;
            long b = bk[i];
            int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long)nbx * nby));
            double hi = o->list_factor * s->h[i];
            double xi[3] = { s->x[i], s->y[i], s->z[i] };
            size_t c = 0;
            int32_t *out = pass ? L->idx + L->start[i] : NULL;
            for (size_t q = bstart[b]; q < bstart[b + 1]; q++) {
                if (out) out[c] = bidx[q];
                c++;
            }
            for (int dx = -1; dx <= 1; dx++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dz = -1; dz <= 1; dz++) {
                        if (!dx && !dy && !dz) continue;
                        int cx = bx + dx, cy = by + dy, cz = bz + dz;
                        if (cx < 0 || cx >= nbx || cy < 0 || cy >= nby || cz < 0 || cz >= nbz) continue;
                        long nb_ = ((long)cz * nby + cy) * nbx + cx;
                        for (size_t q = bstart[nb_]; q < bstart[nb_ + 1]; q++) {
                            int32_t j = bidx[q];
                            double ds[3] = { xi[0] - s->x[j], xi[1] - s->y[j], xi[2] - s->z[j] };
                            if (in_support(ds, hi, 3)) {
                                if (out) out[c] = j;
                                c++;
                            }
                        }
                    }
            if (!pass) cnt[i] = c;
        }
        if (!pass) {
            L->start[0] = 0;
            for (size_t i = 0; i < n; i++) L->start[i + 1] = L->start[i] + cnt[i];
            L->nidx = L->start[n];
            L->idx = (int32_t *)malloc(sizeof(int32_t) * (L->nidx ? L->nidx : 1));
        }
    }
    free(cnt);
    free(is_t);
    free(bk);
    free(bstart);
    free(bidx);
    return PLUME_OK;
}

/* list access: 1D lists hold every particle in creation order
 * (add_air.cc:470-479), 3D lists come from build_lists_3d */
#define FOR_LIST(L, D, n, i, jv, ...)                                         \
    do {                                                                       \
        if ((D) == 1) {                                                        \
            for (size_t q_ = 0; q_ < (n); q_++) { size_t jv = q_; __VA_ARGS__ }\
        } else {                                                               \
            for (size_t q_ = (L)->start[i]; q_ < (L)->start[(i) + 1]; q_++) {  \
                size_t jv = (size_t)(L)->idx[q_]; __VA_ARGS__                  \
            }                                                                  \
        }                                                                      \
    } while (0)

static inline void coords(const PlumeSoA *s, size_t i, int D, double *x)
{
    x[0] = s->x[i];
    if (D == 3) { x[1] = s->y[i]; x[2] = s->z[i]; }
}
static inline void vel(const PlumeSoA *s, size_t i, int D, int smoothed, double *v)
{
    if (smoothed) {
        v[0] = s->vsx[i];
        if (D == 3) { v[1] = s->vsy[i]; v[2] = s->vsz[i]; }
    } else {
        v[0] = s->vx[i];
        if (D == 3) { v[1] = s->vy[i]; v[2] = s->vz[i]; }
    }
}

/* ------------------------------------------------------------------ */
/* adaptive_sml, neighs.cc:479-693 (ADAPTIVE_SML == 1)                  */
/* ------------------------------------------------------------------ */
static int adaptive_pass(const PlumeOptions *o, PlumeSoA *s, size_t n,
                         const Lists *L, int nthreads, size_t ntarget)
{
    const int D = o->dim;
    int err = PLUME_OK;
    size_t seen = 0;
    (void)seen;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long ii = 0; ii < (long)n; ii++) {
        size_t i = (size_t)ii;
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue; /* not a target */
        double xi[3];
        coords(s, i, D, xi);
        for (int loop = 0; loop < o->num_loop; loop++) {
            double H_old = s->h[i];
            double H_star = H_old * o->c_smooth;
            double supp = o->cutoff2 * H_star;
            double rho_star = 0.;
            FOR_LIST(L, D, n, i, j, {
                if (contr_dens(s->bc_type[j], o->pghost_contrib)) {
                    double xj[3], dx[3], si[3];
                    coords(s, j, D, xj);
                    for (int k = 0; k < D; k++) {
                        dx[k] = xi[k] - xj[k];
                        si[k] = dx[k] / H_star;
                    }
                    if (in_support(dx, supp, D)) {
                        double mj = s->mass[j];
                        double wght = kw(o->kernel, si, H_star, D);
                        rho_star += wght * mj;
                    }
                }
            });
            double H_new;
            if (D == 3)
                H_new = o->eta_smooth * cbrt(s->mass[i] / rho_star);
            else
                H_new = o->eta_smooth * (s->mass[i] / rho_star);
            s->h[i] = 1.0 * H_new; /* put_smlen: RATIO_SML_DX * h */
            if (!(H_new > 0) || !isfinite(H_new)) {
#pragma omp critical
                err = PLUME_E_NONPOSITIVE;
                break;
            }
            double errv = fabs((H_new - H_old) / H_old);
            if (errv < o->thresh) break;
        }
    }
    (void)ntarget;
    return err;
}

/* ------------------------------------------------------------------ */
/* mom_engr_update (USE_GSPH == 0), mom_engr_update.cc:29-439           */
/* ------------------------------------------------------------------ */
typedef struct Work {
    double *nv[3], *ne, *nrho, *nY, *nE;
} Work;

static int momentum_pass(const PlumeOptions *o, PlumeSoA *s, size_t n,
                         const Lists *L, double dt, Work *w, int nthreads)
{
    const int D = o->dim;
    const double grav = -o->g; /* gravity[DIMENSION-1], mom_engr_update.cc:53-59 */
    int err = PLUME_OK;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long ii = 0; ii < (long)n; ii++) {
        size_t i = (size_t)ii;
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        double xi[3], veli[3], rhs_v[3] = { 0, 0, 0 }, rhs_e = 0;
        coords(s, i, D, xi);
        double hi = s->h[i];
        double supp = o->cutoff2 * hi;
        double pressi = s->p[i];
        double tempi = s->T[i];
        double Cp_i = s->cp[i];
        if (!(s->rho[i] > 0)) {
#pragma omp critical
            err = PLUME_E_NONPOSITIVE;
            continue;
        }
        double Vi = 1.0 / s->rho[i];
        double pvsqi = pressi * Vi * Vi;
        vel(s, i, D, o->lans, veli);
        FOR_LIST(L, D, n, i, j, {
            if (j != i) {
                double xj[3], dx[3], si[3], dist_sq = 0;
                coords(s, j, D, xj);
                double h = 0.5 * (hi + s->h[j]);
                for (int k = 0; k < D; k++) {
                    dx[k] = xi[k] - xj[k];
                    si[k] = dx[k] / h;
                    dist_sq += dx[k] * dx[k];
                }
                if (in_support(dx, supp, D)) {
                    double mj = s->mass[j];
                    double pressj = s->p[j];
                    double Vj = 1.0 / s->rho[j];
                    double velj[3], velij[3], dwdxi[3];
                    vel(s, j, D, o->lans, velj);
                    for (int k = 0; k < D; k++) velij[k] = veli[k] - velj[k];
                    double rhoab = 0.5 * (s->rho[i] + s->rho[j]);
                    double sndspdab = 0.5 * (s->c[i] + s->c[j]);
                    double vis = art_vis(o, rhoab, sndspdab, dx, velij, dist_sq, h, D);
                    if (o->lans) vis -= eps_mom(velij, Vj, D);
                    double mpvsqij = mj * (pressj * Vj * Vj + pvsqi + vis);
                    for (int k = 0; k < D; k++) dwdxi[k] = kdw(o->kernel, si, h, k, D);
                    double heat_tran = 0.;
                    if (o->lans) {
                        double Cp_ij = 0.5 * (s->cp[j] + Cp_i);
                        double hab = 0.5 * (hi + s->h[j]);
                        double kij = eps_heat(Cp_ij, dx, velij, hab, sndspdab, D);
                        double Fij = compute_F(dwdxi, dx, D);
                        heat_tran = mj * Vj * Vi * kij * (tempi - s->T[j]) * Fij;
                    }
                    for (int k = 0; k < D; k++) rhs_v[k] -= mpvsqij * dwdxi[k];
                    double deltae = 0.;
                    for (int k = 0; k < D; k++) deltae += 0.5 * (mpvsqij * dwdxi[k]) * velij[k];
                    rhs_e += (deltae + heat_tran);
                }
            }
        });
        double vi[3];
        vel(s, i, D, 0, vi);
        double unew[3];
        for (int k = 0; k < D; k++) unew[k] = vi[k] + dt * (rhs_v[k]);
        unew[D - 1] += dt * grav;
        for (int k = 0; k < D; k++) w->nv[k][i] = unew[k];
        w->ne[i] = s->e[i] + dt * (rhs_e + veli[D - 1] * grav);
    }
    if (err) return err;
    /* commit loop, mom_engr_update.cc:412-432 */
    for (size_t i = 0; i < n; i++) {
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        s->vx[i] = w->nv[0][i];
        if (D == 3) { s->vy[i] = w->nv[1][i]; s->vz[i] = w->nv[2][i]; }
        s->e[i] = w->ne[i];
        eos(o, s, i);
    }
    return PLUME_OK;
}

/* ------------------------------------------------------------------ */
/* GSPH (USE_GSPH 1)                                                    */
/* ------------------------------------------------------------------ */
/* Gradients (calc_gradients, calculate_gradient.cc:22-208) of rho, the D
 * velocity components and p of every particle with a list: the SPH sums
 * A_ab = -sum_j dx_a (m_j/rho_j) dW_b(dx/h_i, h_i) and
 * F_a,q = -sum_j (f_q,i - f_q,j) (m_j/rho_j) dW_a over the list entries
 * j != i inside the CUTOFF2*h_i box; grad = linsolve(A, F) when more than
 * 20 entries were inside the box, else zero.  linsolve (sph_lib.cc:
 * 161-182) multiplies F by inv3(A) in 3D and by inv1(A) = -1/A in 1D (the
 * reference's sign).  Layout: grad[i*NQ*D + q*D + k], q = rho, v_0..v_D-1,
 * p. */
static void gsph_gradients(const PlumeOptions *o, const PlumeSoA *s, size_t n,
                           const Lists *L, double *grad, int nthreads)
{
    const int D = o->dim, NQ = D + 2;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long ii = 0; ii < (long)n; ii++) {
        size_t i = (size_t)ii;
        double *gi = grad + i * (size_t)(NQ * D);
        for (int q = 0; q < NQ * D; q++) gi[q] = 0.0;
        /* 1D lists belong to the need_neigh particles only (add_air.cc:470-479) */
        if (D == 1 && !need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        double xi[3], vi[3], AA[9] = { 0 }, FF[3][5] = { { 0 } };
        coords(s, i, D, xi);
        vel(s, i, D, 0, vi);
        double hi = s->h[i], supp = o->cutoff2 * hi;
        int nreal = 0;
        FOR_LIST(L, D, n, i, j, {
            if (j != i) {
                double xj[3], dx[3], sv[3];
                coords(s, j, D, xj);
                for (int k = 0; k < D; k++) dx[k] = xi[k] - xj[k];
                if (in_support(dx, supp, D)) {
                    nreal++;
                    double dwm[3], vj[3];
                    for (int k = 0; k < D; k++) sv[k] = dx[k] / hi;
                    for (int k = 0; k < D; k++) dwm[k] = d_weight_gauss(sv, hi, k, D) * s->mass[j] / s->rho[j];
                    for (int a = 0; a < D; a++)
                        for (int b = 0; b < D; b++) AA[a * D + b] -= dx[a] * dwm[b];
                    vel(s, j, D, 0, vj);
                    for (int a = 0; a < D; a++) {
                        FF[a][0] -= (s->rho[i] - s->rho[j]) * dwm[a];
                        for (int b = 0; b < D; b++) FF[a][b + 1] -= (vi[b] - vj[b]) * dwm[a];
                        FF[a][NQ - 1] -= (s->p[i] - s->p[j]) * dwm[a];
                    }
                }
            }
        });
        if (nreal <= 20) continue;
        double Ai[9];
        if (D == 1) {
            Ai[0] = -1 / AA[0];
        } else {
            /* inv3 (sph_lib.cc:86-110) returns the cofactor matrix over the
             * determinant, entry (a,b) = C_ab: the inverse of A transposed,
             * which is the inverse here since A is symmetric */
            double C[9];
            C[0] = AA[4] * AA[8] - AA[5] * AA[7];
            C[1] = -(AA[3] * AA[8] - AA[5] * AA[6]);
            C[2] = AA[3] * AA[7] - AA[4] * AA[6];
            C[3] = -(AA[1] * AA[8] - AA[2] * AA[7]);
            C[4] = AA[0] * AA[8] - AA[2] * AA[6];
            C[5] = -(AA[0] * AA[7] - AA[1] * AA[6]);
            C[6] = AA[1] * AA[5] - AA[2] * AA[4];
            C[7] = -(AA[0] * AA[5] - AA[2] * AA[3]);
            C[8] = AA[0] * AA[4] - AA[1] * AA[3];
            double id = 1.0 / (AA[0] * C[0] + AA[1] * C[1] + AA[2] * C[2]);
            for (int q = 0; q < 9; q++) Ai[q] = C[q] * id;
        }
        /* ff = Ai F (matrix_matrix_mult, sph_lib.cc:136-156); gradU[q*D+a] = ff[a][q] */
        for (int a = 0; a < D; a++)
            for (int q = 0; q < NQ; q++) {
                double acc = 0.0;
                for (int b = 0; b < D; b++) acc += Ai[a * D + b] * FF[b][q];
                gi[q * D + a] = acc;
            }
    }
}

/* HLLC Riemann solver of the GSPH step (HLLC_RP_Solver, sph_lib.cc:
 * 1753-1908, HLL_WAVE_SPEED_EVA 0, USE_GSPH 1): Roe-averaged interface
 * state, wave speeds S_l = min(v_l - c_l, -c_lr), S_r = max(v_r + c_r, c_lr)
 * relative to the Roe velocity, contact speed S_m; returns p* and u* of the
 * region that contains the interface.  l is particle j's side, r particle
 * i's. */
static void hllc(double dl, double dr, double pl, double pr, double ul, double ur, double gl, double gr,
                 double *p_star, double *u_star)
{
    double rdl = sqrt(dl), rdr = sqrt(dr);
    double den = 1.0 / (rdl + rdr);
    double ulr = (ul * rdl + ur * rdr) * den;
    double plr = (pl * rdl + pr * rdr) * den;
    double glr = (gl * rdl + gr * rdr) * den;
    double dlr = (dl * rdl + dr * rdr) * den;
    double clr = sqrt(glr * plr / dlr);
    double vl = ul - ulr, vr = ur - ulr;
    double cl = sqrt(gl * pl / dl), cr = sqrt(gr * pr / dr);
    double Sl = fmin(vl - cl, -clr);
    double Sr = fmax(vr + cr, clr);
    double Sm = (dr * vr * (Sr - vr) - dl * vl * (Sl - vl) + pl - pr) / (dr * (Sr - vr) - dl * (Sl - vl));
    double ph = dl * (vl - Sl) * (vl - Sm) + pl;
    double Ml = dl * ul, Mr = dr * ur;
    double El = dl * (pl / (dl * (gl - 1)) + 0.5 * ul * ul);
    double Er = dr * (pr / (dr * (gr - 1)) + 0.5 * ur * ur);
    if (Sl > 0) {
        *p_star = pl;
        *u_star = ul;
    } else if (Sl <= 0 && Sm > 0) {
        *p_star = Sm / (Sl - Sm) * ((Sl - vl) * Ml + (ph - pl)) + ph;
        *u_star = (Sm / (Sl - Sm) * ((Sl - vl) * El + ph * Sm - pl * vl) + (Sm + ulr) * ph) / (*p_star);
    } else if (Sm <= 0 && Sr > 0) {
        *p_star = Sm / (Sr - Sm) * ((Sr - vr) * Mr + (ph - pr)) + ph;
        *u_star = (Sm / (Sr - Sm) * ((Sr - vr) * Er + ph * Sm - pr * vr) + (Sm + ulr) * ph) / (*p_star);
    } else if (Sr <= 0) {
        *p_star = pr;
        *u_star = ur;
    } else {
        /* a NaN wave speed: the reference leaves p*, u* unset */
        *p_star = NAN;
        *u_star = NAN;
    }
}

/* Roe Riemann solver (Roe_RP_Solver, sph_lib.cc:1694-1750, RP_MASS_WEIGHTED
 * 0, FLUID_COMPRESSIBILITY 0): Roe averages, the Lagrangian sound speed
 * rho_lr c_lr, p* = p_lr - c/2 (u_r - u_l), u* = u_lr - (p_r - p_l)/(2c). */
static void roe(double dl, double dr, double pl, double pr, double ul, double ur, double gl, double gr,
                double *p_star, double *u_star)
{
    double rdl = sqrt(dl), rdr = sqrt(dr);
    double den = 1.0 / (rdl + rdr);
    double plr = (pl * rdl + pr * rdr) * den;
    double glr = (gl * rdl + gr * rdr) * den;
    double dlr = (dl * rdl + dr * rdr) * den;
    double clr = sqrt(glr * plr / dlr);
    clr = dlr * clr;
    double ulr = (ul * rdl + ur * rdr) * den;
    *p_star = plr - 0.5 * clr * (ur - ul);
    *u_star = ulr - 0.5 * (pr - pl) / clr;
}

/* HLLC_RP_Solver_my (sph_lib.cc:1912-2088): HLLC for strong shocks on the
 * velocities relative to the Roe velocity; wave speeds by HLL_WAVE_SPEED_EVA
 * (2 Davis, 3 Toro); the star region takes p_HLLC and u = sqrt(2 (E*_l -
 * e*_l)), the outer regions the side's state. */
static void hllc_my(int wave, double dl, double dr, double pl, double pr, double ul, double ur,
                    double gl, double gr, double *p_star, double *u_star)
{
    double rdl = sqrt(dl), rdr = sqrt(dr);
    double den = 1.0 / (rdl + rdr);
    double cl = sqrt(gl * pl / dl), cr = sqrt(gr * pr / dr);
    double ulr = (ul * rdl + ur * rdr) * den;
    ul = ul - ulr;
    ur = ur - ulr;
    double Sl, Sr;
    if (wave == 2) {
        Sl = fmin(ul - cl, ur - cr);
        Sr = fmax(ul + cl, ur + cr);
    } else {
        double plr = (pl * rdl + pr * rdr) * den;
        double glr = (gl * rdl + gr * rdr) * den;
        double dlr = (dl * rdl + dr * rdr) * den;
        double clr = sqrt(glr * plr / dlr);
        double p_refs = fmax(0.0, 0.5 * (pl + pr) + 0.25 * (ul - ur) * (dr + dl) * clr);
        double ql = p_refs < pl ? 1.0 : sqrt(1.0 + 0.5 * (gl + 1.0) / gl * (p_refs / pl - 1.0));
        double qr = p_refs < pr ? 1.0 : sqrt(1.0 + 0.5 * (gr + 1.0) / gr * (p_refs / pr - 1.0));
        Sl = ul - cl * ql;
        Sr = ur + cr * qr;
    }
    double alf_l = dl * (Sl - ul), alf_r = dr * (Sr - ur);
    double Sm = (ur * alf_r - ul * alf_l + pl - pr) / (alf_r - alf_l);
    double p_hllc = (pr * alf_r - pl * alf_l - alf_r * alf_l * (ul - ur)) / (alf_r - alf_l);
    double dl_star = alf_l / (Sl - Sm);
    double el_star = p_hllc / (dl_star * (gl - 1.0));
    double el = pl / (dl * (gl - 1.0));
    double El_star = el + (Sm - ul) * (Sm + pl / alf_l);
    double u_hllc = sqrt(2.0 * (El_star - el_star));
    if (Sl > 0) {
        *p_star = pl;
        *u_star = ul;
    } else if (Sl <= 0 && Sr > 0) {
        *p_star = p_hllc;
        *u_star = u_hllc;
    } else if (Sr <= 0) {
        *p_star = pr;
        *u_star = ur;
    } else {
        /* a NaN wave speed: the reference leaves p*, u* unset */
        *p_star = NAN;
        *u_star = NAN;
    }
}

/* VanLeer_RP_Solver (sph_lib.cc:2094-2210): Van Leer's iterative solver on
 * the Lagrangian sound speeds C = rho c of the particles' own sound speeds:
 * the acoustic estimate of p*, accepted within 1 % of both pressures, else
 * iterated with the shock / rarefaction impedances W and slopes Z until p*
 * moves by less than 1 % (at most PLUME_VANLEER_MAX_ITER iterations, then
 * NaN; the reference iterates without a limit). */
static void vanleer(double dl, double dr, double pl, double pr, double ul, double ur, double gl,
                    double gr, double csl, double csr, double *p_star, double *u_star)
{
    double Cl = csl * dl, Cr = csr * dr;
    double p = (Cl * pr + Cr * pl - Cr * Cl * (ul - ur)) / (Cl + Cr);
    double md = fabs(p - pl) / pl, md2 = fabs(p - pr) / pr;
    if (md2 > md) md = md2;
    if (md < 0.01) {
        *u_star = 0.5 * (ul + ur);
        *p_star = p;
        return;
    }
    double G1l = 0.5 * (gl + 1) / gl, G2l = 0.5 * (gl - 1) / gl, G3l = 1.0 - G2l;
    double G1r = 0.5 * (gr + 1) / gr, G2r = 0.5 * (gr - 1) / gr, G3r = 1.0 - G2r;
    double Cl2 = Cl * Cl, Cr2 = Cr * Cr;
    double Zl = 0, Zr = 0, vl = 0, vr = 0, err = 1.0;
    int it = 0;
    while (err > 0.01) {
        if (++it > PLUME_VANLEER_MAX_ITER) {
            *p_star = NAN;
            *u_star = NAN;
            return;
        }
        double Rl = p / pl, Rr = p / pr;
        double Wl = (p >= pl) ? Cl * pow(1.0 + G1l * (p - pl) / pl, 0.5)
                              : G2l * (1.0 - Rl) / (1.0 - pow(Rl, G2l)) * Cl;
        double Wr = (p >= pr) ? Cr * pow(1.0 + G1r * (p - pr) / pr, 0.5)
                              : G2r * (1.0 - Rr) / (1.0 - pow(Rr, G2r)) * Cr;
        double Wl2 = Wl * Wl, Wr2 = Wr * Wr;
        Zl = (p >= pl) ? 2.0 * Wl2 / (Wl2 + Cl2) * Wl : Cl * pow(Rl, G3l);
        Zr = (p >= pr) ? 2.0 * Wr2 / (Wr2 + Cr2) * Wr : Cr * pow(Rr, G3r);
        vl = ul + (p - pl) / Wl;
        vr = ur - (p - pr) / Wr;
        double pn = p - (Zl * Zr * (vl - vr)) / (Zl + Zr);
        err = fabs(pn - p) / p;
        p = pn;
    }
    *u_star = (Zl * vl + Zr * vr) / (Zl + Zr);
    *p_star = p;
}

/* Generate_VanderCorput (sph_lib.cc:2214-2245): n brought below 65,537 by
 * steps of 65,536, bits 0..15 of n mirrored about the binary point */
static double vdc16(unsigned n)
{
    while (n > 65536u) n -= 65536u;
    double v = 0.0, w = 0.5;
    for (int k = 0; k < 16; k++) {
        if (n & (1u << k)) v += w;
        w *= 0.5;
    }
    return v;
}

/* HLLC_RP_Solver under USE_GSPH 2 (sph_lib.cc:1753-1885): the waves of
 * hllc(), the solution sampled at x = 0.6 (sp - 1/2) dist against the waves'
 * positions S dt (random choice method) */
static void hllc_rcm(double dl, double dr, double pl, double pr, double ul, double ur, double gl, double gr,
                     double sp, double dt, double dist, double *p_star, double *u_star)
{
    double rdl = sqrt(dl), rdr = sqrt(dr);
    double den = 1.0 / (rdl + rdr);
    double ulr = (ul * rdl + ur * rdr) * den;
    double plr = (pl * rdl + pr * rdr) * den;
    double glr = (gl * rdl + gr * rdr) * den;
    double dlr = (dl * rdl + dr * rdr) * den;
    double clr = sqrt(glr * plr / dlr);
    double vl = ul - ulr, vr = ur - ulr;
    double cl = sqrt(gl * pl / dl), cr = sqrt(gr * pr / dr);
    double Sl = fmin(vl - cl, -clr);
    double Sr = fmax(vr + cr, clr);
    double Sm = (dr * vr * (Sr - vr) - dl * vl * (Sl - vl) + pl - pr) / (dr * (Sr - vr) - dl * (Sl - vl));
    double ph = dl * (vl - Sl) * (vl - Sm) + pl;
    double Ml = dl * ul, Mr = dr * ur;
    double El = dl * (pl / (dl * (gl - 1)) + 0.5 * ul * ul);
    double Er = dr * (pr / (dr * (gr - 1)) + 0.5 * ur * ur);
    double xSl = Sl * dt, xSm = Sm * dt, xSr = Sr * dt;
    double x = (sp - 0.5) * dist * 0.6;
    if (xSl > x) {
        *p_star = pl;
        *u_star = ul;
    } else if (xSl <= x && xSm > x) {
        *p_star = Sm / (Sl - Sm) * ((Sl - vl) * Ml + (ph - pl)) + ph;
        *u_star = (Sm / (Sl - Sm) * ((Sl - vl) * El + ph * Sm - pl * vl) + (Sm + ulr) * ph) / (*p_star);
    } else if (xSm <= x && xSr > x) {
        *p_star = Sm / (Sr - Sm) * ((Sr - vr) * Mr + (ph - pr)) + ph;
        *u_star = (Sm / (Sr - Sm) * ((Sr - vr) * Er + ph * Sm - pr * vr) + (Sm + ulr) * ph) / (*p_star);
    } else if (xSr <= x) {
        *p_star = pr;
        *u_star = ur;
    } else {
        *p_star = NAN;
        *u_star = NAN;
    }
}

/* One pair's Riemann problem (Riemann_Solver, sph_lib.cc:2247-2598, USE_GSPH
 * 1, RP_MASS_WEIGHTED 0, SWITCH_OFF_AV_FOR_EXPAN 0, SHEAR_VEL_APP 2): the
 * states projected on e = (x_i - x_j)/|x_i - x_j|; unless the
 * reconstruction is zeroth order, the gradients projected on e, limited
 * (monotonicity: opposite velocity slopes, or C_SHOCK (u_j - u_i) -- its
 * absolute value under the modified condition -- above the smaller sound
 * speed), the interface placed at s* (GSPH_SPECIFIC_VOL_APP 0: midpoint;
 * 1, 3: Compute_sij_star, sph_lib.cc:1655-1692) and the states moved to it
 * over c dt/2 with the MINI_DERIVATIVE_COND fallback; the Roe or HLLC
 * solution u* put back along e with the Roe-averaged transverse velocity. */
typedef struct GsphSide {
    double rho, p, c, gam, h;
    const double *v;   /* velocity used by the step (smoothed under LANS) */
    const double *g;   /* gradients (rho, v, p) x D, NULL when not computed */
} GsphSide;

static void gsph_riemann(const PlumeOptions *o, int D, const double *xi, const double *xj,
                         const GsphSide *I, const GsphSide *J, double dt_half,
                         double *p_star, double *v_star, double sp)
{
    const int rcm = o->method == PLUME_METHOD_GSPH_RCM;  /* USE_GSPH 2 */
    double dx[3], e[3], dist = 0.0;
    for (int k = 0; k < D; k++) dx[k] = xi[k] - xj[k];
    for (int k = 0; k < D; k++) dist += dx[k] * dx[k];
    dist = sqrt(dist);
    for (int k = 0; k < D; k++) e[k] = dx[k] / dist;
    double ui = 0.0, uj = 0.0;
    for (int k = 0; k < D; k++) {
        ui += I->v[k] * e[k];
        uj += J->v[k] * e[k];
    }
    const int recon = o->gsph_recon;
    double dr = I->rho, ur = ui, pr = I->p, dl = J->rho, ul = uj, pl = J->p;
    if (recon != PLUME_RECON_ZEROTH) {
        const int NQ = D + 2;
        const double z3[15] = { 0 };
        const double *gi = I->g ? I->g : z3, *gj = J->g ? J->g : z3;
        double drhoi = 0, dpi = 0, drhoj = 0, dpj = 0, dv_i[3] = { 0, 0, 0 }, dv_j[3] = { 0, 0, 0 };
        for (int k = 0; k < D; k++) {
            drhoi += gi[0 * D + k] * e[k];
            drhoj += gj[0 * D + k] * e[k];
            dpi += gi[(NQ - 1) * D + k] * e[k];
            dpj += gj[(NQ - 1) * D + k] * e[k];
            for (int c = 0; c < D; c++) {
                dv_i[c] += gi[(1 + c) * D + k] * e[k];
                dv_j[c] += gj[(1 + c) * D + k] * e[k];
            }
        }
        double ddui = 0.0, dduj = 0.0;
        for (int c = 0; c < D; c++) {
            ddui += dv_i[c] * e[c];
            dduj += dv_j[c] * e[c];
        }
        if (ddui * dduj < 0) ddui = dduj = 0.0;
        double du = uj - ui;
        if (o->gsph_mono) du = fabs(du);
        if (OR_C_SHOCK * du > fmin(I->c, J->c)) drhoi = dpi = ddui = drhoj = dpj = dduj = 0.0;
        double Si = 0.5 * dist, Sj = -Si, sij = 0.0;
        const double hij = 0.5 * (I->h + J->h), Vi = 1 / I->rho, Vj = 1 / J->rho;
        if (o->gsph_vol == 1) {
            double Cc = (Vi - Vj) / dist, Dd = (Vi + Vj) * 0.5, hsq = hij * hij;
            double Vsq = 0.25 * hsq * Cc * Cc + Dd * Dd;
            sij = 0.5 * (hsq * Cc * Dd) / Vsq;
        } else if (o->gsph_vol == 3) {
            double DVi = -Vi * Vi * drhoi, DVj = -Vj * Vj * drhoj;
            double d2 = dist * dist, d3 = d2 * dist;
            double A = -2.0 * (Vi - Vj) / d3 + (DVi + DVj) / d2;
            double B = 0.5 * (DVi - DVj) / dist;
            double Cc = 1.5 * (Vi - Vj) / dist - 0.25 * (DVi + DVj);
            double Dd = 0.5 * (Vi + Vj) - 0.125 * (DVi - DVj) * dist;
            double hsq = hij * hij, h4 = hsq * hsq, h6 = h4 * hsq;
            double Vsq = 0.234375 * h6 * A * A + 0.1875 * h4 * (2.0 * A * Cc + B * B) +
                         0.25 * hsq * (2.0 * B * Dd + Cc * Cc) + Dd * Dd;
            sij = (0.46875 * h6 * A * B + 0.375 * h4 * (A * Dd + B * Cc) + 0.5 * hsq * Cc * Dd) / Vsq;
        }
        if (rcm) sij = (sp - 0.5) * dist;
        double delta_i = sij + I->c * dt_half - Si;
        double delta_j = sij - J->c * dt_half - Sj;
        dr = I->rho + drhoi * delta_i;
        ur = ui + ddui * delta_i;
        pr = I->p + dpi * delta_i;
        dl = J->rho + drhoj * delta_j;
        ul = uj + dduj * delta_j;
        pl = J->p + dpj * delta_j;
        if (recon == PLUME_RECON_ALL) {
            if (dr < 0 || dl < 0 || pr < 0 || pl < 0) {
                dr = I->rho; ur = ui; pr = I->p; dl = J->rho; ul = uj; pl = J->p;
            }
        } else if (recon == PLUME_RECON_PAIRWISE) {
            if (dr < 0 || dl < 0) { dr = I->rho; dl = J->rho; }
            if (pr < 0 || pl < 0) { pr = I->p; pl = J->p; }
        } else if (recon == PLUME_RECON_EACH || recon == PLUME_RECON_EACH_SHOCK) {
            if (dr < 0) dr = I->rho;
            if (dl < 0) dl = J->rho;
            if (pr < 0) pr = I->p;
            if (pl < 0) pl = J->p;
            if (recon == PLUME_RECON_EACH_SHOCK && 3.0 * fabs(ul - ur) > fmin(I->c, J->c)) {
                ul = uj;
                ur = ui;
            }
        }
    }
    double u_star;
    if (rcm)
        hllc_rcm(dl, dr, pl, pr, ul, ur, J->gam, I->gam, sp, 2.0 * dt_half, dist, p_star, &u_star);
    else if (o->gsph_solver == PLUME_RIEMANN_HLLC)
        hllc(dl, dr, pl, pr, ul, ur, J->gam, I->gam, p_star, &u_star);
    else if (o->gsph_solver == PLUME_RIEMANN_HLLC_MY)
        hllc_my(o->gsph_wave_speed, dl, dr, pl, pr, ul, ur, J->gam, I->gam, p_star, &u_star);
    else if (o->gsph_solver == PLUME_RIEMANN_VANLEER)
        vanleer(dl, dr, pl, pr, ul, ur, J->gam, I->gam, J->c, I->c, p_star, &u_star);
    else
        roe(dl, dr, pl, pr, ul, ur, J->gam, I->gam, p_star, &u_star);
    double rdl = sqrt(dl), rdr = sqrt(dr);
    double den = 1.0 / (rdl + rdr);
    double ulr = (ul * rdl + ur * rdr) * den;
    for (int k = 0; k < D; k++) {
        double vlr = (J->v[k] * rdl + I->v[k] * rdr) * den;
        v_star[k] = e[k] * u_star + vlr - ulr * e[k];
    }
}

/* GSPH momentum and energy (mom_engr_update.cc:441-1146, ME_UPDATE_SML 2,
 * ADAPTIVE_SML 1, HAVE_ENERGY_CUT 0): per need_neigh particle two passes
 * over its list entries j != i inside the CUTOFF2*h_i box whose
 * V_i^2 dW(dx/h_ij, h_ij) is non-zero (h_ij = (h_i+h_j)/2):
 *   pass 1: rhs_v -= m_j (p* (V_i^2 + V_j^2) dW - tau dW), tau the LANS
 *           stress SPH_epsilon_mom(v_i - v_j, V_j) (0 without LANS);
 *   pass 2: the same Riemann problems again, rhs_e -= m_j (v* - xdot*) .
 *           (p* (V_i^2 + V_j^2) dW - tau dW) + the LANS heat flux, with
 *           xdot* = v_i + dt/2 (rhs_v + g);
 * then v += dt (rhs_v + g e_D), e += dt (rhs_e + v_i,D g), and the commit
 * with the EOS.  grad: the gradients of gsph_gradients or NULL. */
static int gsph_momentum_pass(const PlumeOptions *o, PlumeSoA *s, size_t n, const Lists *L,
                              double dt, const double *grad, Work *w, int nthreads, int step)
{
    /* random choice method: the step's sample point (mom_engr_update.cc:513-516) */
    const double sp = o->method == PLUME_METHOD_GSPH_RCM ? vdc16((unsigned)step) : 0.5;
    const int D = o->dim, NQ = D + 2;
    const double grav = -o->g;
    const double dt_half = 0.5 * dt;
    int err = PLUME_OK;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long ii = 0; ii < (long)n; ii++) {
        size_t i = (size_t)ii;
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        double xi[3], veli[3], rhs_v[3] = { 0, 0, 0 }, rhs_e = 0;
        coords(s, i, D, xi);
        double hi = s->h[i];
        double supp = o->cutoff2 * hi;
        if (!(s->rho[i] > 0)) {
#pragma omp critical
            err = PLUME_E_NONPOSITIVE;
            continue;
        }
        double Vi = 1.0 / s->rho[i];
        vel(s, i, D, o->lans, veli);
        GsphSide I = { s->rho[i], s->p[i], s->c[i], s->gamma[i], hi, veli,
                       grad ? grad + i * (size_t)(NQ * D) : NULL };
        for (int pass = 0; pass < 2; pass++) {
            double xdot[3];
            for (int k = 0; k < D; k++) xdot[k] = veli[k] + 0.5 * dt * (rhs_v[k] + (k == D - 1 ? grav : 0.0));
            FOR_LIST(L, D, n, i, j, {
                if (j != i) {
                    double xj[3], dx[3], si[3];
                    coords(s, j, D, xj);
                    for (int k = 0; k < D; k++) dx[k] = xi[k] - xj[k];
                    if (in_support(dx, supp, D)) {
                        double Vj = 1.0 / s->rho[j];
                        double hij = 0.5 * (hi + s->h[j]);
                        double dwdx[3], vsqi[3], vsqj[3], max_dw = 0.0;
                        for (int k = 0; k < D; k++) si[k] = dx[k] / hij;
                        for (int k = 0; k < D; k++) dwdx[k] = d_weight_gauss(si, hij, k, D);
                        for (int k = 0; k < D; k++) {
                            vsqi[k] = Vi * Vi * dwdx[k];
                            vsqj[k] = Vj * Vj * dwdx[k];
                        }
                        for (int k = 0; k < D; k++)
                            if (fabs(vsqi[k]) > max_dw) max_dw = fabs(vsqi[k]);
                        if (max_dw > 0) {
                            double velj[3], velij[3], p_star, v_star[3], tau = 0.0;
                            vel(s, j, D, o->lans, velj);
                            GsphSide J = { s->rho[j], s->p[j], s->c[j], s->gamma[j], s->h[j], velj,
                                           grad ? grad + j * (size_t)(NQ * D) : NULL };
                            gsph_riemann(o, D, xi, xj, &I, &J, dt_half, &p_star, v_star, sp);
                            for (int k = 0; k < D; k++) velij[k] = veli[k] - velj[k];
                            if (o->lans) tau = eps_mom(velij, Vj, D);
                            if (pass == 0) {
                                for (int k = 0; k < D; k++)
                                    rhs_v[k] -= s->mass[j] * (p_star * (vsqi[k] + vsqj[k]) - tau * dwdx[k]);
                            } else {
                                double heat = 0.0;
                                if (o->lans) {
                                    double rhoab = 0.5 * (s->rho[i] + s->rho[j]);
                                    double cab = 0.5 * (s->c[i] + s->c[j]);
                                    double Cp_ij = 0.5 * (s->cp[j] + s->cp[i]);
                                    double hab = 0.5 * (hi + s->h[j]);
                                    (void)rhoab;
                                    double kij = eps_heat(Cp_ij, dx, velij, hab, cab, D);
                                    double Fij = compute_F(dwdx, dx, D);
                                    heat = s->mass[j] * Vj * Vi * kij * (s->T[i] - s->T[j]) * Fij;
                                }
                                double de = 0.0;
                                for (int k = 0; k < D; k++)
                                    de -= s->mass[j] * (v_star[k] - xdot[k]) *
                                          (p_star * (vsqi[k] + vsqj[k]) - tau * dwdx[k]);
                                rhs_e += (de + heat);
                            }
                        }
                    }
                }
            });
        }
        double vi[3];
        vel(s, i, D, 0, vi);
        double unew[3];
        for (int k = 0; k < D; k++) unew[k] = vi[k] + dt * (rhs_v[k]);
        unew[D - 1] += dt * grav;
        for (int k = 0; k < D; k++) w->nv[k][i] = unew[k];
        w->ne[i] = s->e[i] + dt * (rhs_e + veli[D - 1] * grav);
    }
    if (err) return err;
    for (size_t i = 0; i < n; i++) {
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        s->vx[i] = w->nv[0][i];
        if (D == 3) { s->vy[i] = w->nv[1][i]; s->vz[i] = w->nv[2][i]; }
        s->e[i] = w->ne[i];
        eos(o, s, i);
    }
    return PLUME_OK;
}

/* ------------------------------------------------------------------ */
/* smooth_density, density_massfrac.cc:25-359                           */
/* (DENSITY_UPDATE_SML 11, DENSITY_UPDATE_SPH 11, HAVE_ENERGY_SMOOTH)   */
/* ------------------------------------------------------------------ */
static int density_pass(const PlumeOptions *o, PlumeSoA *s, size_t n,
                        const Lists *L, Work *w, int nthreads)
{
    const int D = o->dim;
    int err = PLUME_OK;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long ii = 0; ii < (long)n; ii++) {
        size_t i = (size_t)ii;
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        double xi[3];
        coords(s, i, D, xi);
        double hi0 = s->h[i];
        double supp = o->cutoff2 * hi0;
        double tmprho[2] = { 0., 0. };
        double wnorm_e = 0.0, engr = 0.0;
        FOR_LIST(L, D, n, i, j, {
            if (contr_dens(s->bc_type[j], o->pghost_contrib)) {
                double mj = s->mass[j];
                double rhoj = s->rho[j];
                int ph = s->phase[j];
                if (ph == 1 || ph == 2) {
                    double xj[3], ds[3], sv[3];
                    coords(s, j, D, xj);
                    for (int k = 0; k < D; k++) ds[k] = xi[k] - xj[k];
                    if (in_support(ds, supp, D)) {
                        double hh = 0.5 * (s->h[i] + s->h[j]);
                        for (int k = 0; k < D; k++) sv[k] = ds[k] / hh;
                        if (o->energy_smooth) {
                            double s_e[3];
                            for (int k = 0; k < D; k++) s_e[k] = OR_E_SMOOTH * ds[k] / hh;
                            double wm_e = kw(o->kernel, s_e, hh / OR_E_SMOOTH, D) * mj;
                            wnorm_e += wm_e / rhoj;
                            engr += wm_e * s->e[j] / rhoj;
                        }
                        double wght = kw(o->kernel, sv, hh, D);
                        double wm = wght * mj;
                        tmprho[ph - 1] += wm;
                    }
                }
            }
        });
        double density = 0.0;
        if (o->energy_smooth) {
            if (!(wnorm_e > 0)) {
#pragma omp critical
                err = PLUME_E_NONPOSITIVE;
                continue;
            }
            engr = engr / wnorm_e;
            w->nE[i] = engr;
        }
        density += tmprho[0];
        density += tmprho[1];
        double mssfrc = tmprho[1] / density;
        if (!(density > 0)) {
#pragma omp critical
            err = PLUME_E_NONPOSITIVE;
            continue;
        }
        w->nrho[i] = density;
        w->nY[i] = mssfrc;
    }
    if (err) return err;
    /* commit loop, density_massfrac.cc:337-352 */
    for (size_t i = 0; i < n; i++) {
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        s->Y[i] = w->nY[i];
        if (s->Y[i] >= OR_MSFRC_TH && s->involved[i] != 2) s->involved[i] = 2;
        s->rho[i] = w->nrho[i];
        if (o->energy_smooth) s->e[i] = w->nE[i];
        eos(o, s, i);
    }
    return PLUME_OK;
}

/* ------------------------------------------------------------------ */
/* smooth_velocity, smooth_velocity.cc:25-165 (HAVE_TURBULENCE_LANS 1)   */
/* ------------------------------------------------------------------ */
static int velocity_pass(const PlumeOptions *o, PlumeSoA *s, size_t n,
                         const Lists *L, int nthreads)
{
    const int D = o->dim;
    int err = PLUME_OK;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
    for (long ii = 0; ii < (long)n; ii++) {
        size_t i = (size_t)ii;
        if (!need_neigh(s->bc_type[i])) continue;
        if (D == 3 && L->start[i + 1] == L->start[i]) continue;
        double xi[3], vi[3], temp_dv[3] = { 0, 0, 0 }, wnorm = 0.;
        coords(s, i, D, xi);
        vel(s, i, D, 0, vi);
        double hi = s->h[i];
        double supp = o->cutoff2 * hi;
        FOR_LIST(L, D, n, i, j, {
            if (contr_vel_smooth(s->bc_type[j])) {
                double xj[3], ds[3], sv[3], vj[3];
                coords(s, j, D, xj);
                for (int k = 0; k < D; k++) ds[k] = xi[k] - xj[k];
                if (in_support(ds, supp, D)) {
                    double rhoj = s->rho[j];
                    double mj = s->mass[j];
                    for (int k = 0; k < D; k++) sv[k] = ds[k] / hi;
                    double wght = kw(o->kernel, sv, hi, D);
                    double mvw = wght * mj / rhoj;
                    vel(s, j, D, 0, vj);
                    for (int k = 0; k < D; k++) temp_dv[k] += mvw * (vj[k] - vi[k]);
                    wnorm += mvw;
                }
            }
        });
        if (!(wnorm > 0)) {
#pragma omp critical
            err = PLUME_E_NONPOSITIVE;
            continue;
        }
        for (int k = 0; k < D; k++) temp_dv[k] /= wnorm;
        s->vsx[i] = vi[0] + temp_dv[0];
        if (D == 3) {
            s->vsy[i] = vi[1] + temp_dv[1];
            s->vsz[i] = vi[2] + temp_dv[2];
        }
    }
    return err;
}

/* ------------------------------------------------------------------ */
/* timestep, timestep.cc:94-135 (3D) and :139-183 (1D)                  */
/* ------------------------------------------------------------------ */
static int timestep(const PlumeOptions *o, const PlumeSoA *s, size_t n, double *out)
{
    double dt = 1.0E+10;
    for (size_t i = 0; i < n; i++) {
        if (!need_neigh(s->bc_type[i])) continue;
        double c = s->c[i];
        if (!(c > 0)) return PLUME_E_NONPOSITIVE;
        double temp = s->h[i] / c;
        if (temp < dt) dt = temp;
    }
    *out = o->cfl * dt;
    return PLUME_OK;
}

/* TimeProps::incrtime, properties.h:71-83 */
static void incrtime(const PlumeOptions *o, OracleTime *t, double *dt)
{
    if ((t->time + (*dt)) > t->ndtimeoutput) (*dt) = t->ndtimeoutput - t->time;
    if ((t->time + (*dt)) > o->max_time) (*dt) = o->max_time - t->time;
    t->time += (*dt);
    t->dtime = (*dt);
    t->step++;
}
/* TimeProps::ifoutput, properties.h:100-118 */
static void ifoutput(const PlumeOptions *o, OracleTime *t)
{
    if (t->time >= t->ndtimeoutput || t->time == o->max_time) {
        t->ioutput++;
        t->ndtimeoutput = ((t->ioutput + 1) * o->timeoutput) / 1.0;
    }
}
/* TimeProps::iferupt, properties.h:123-131 */
static int iferupt(const PlumeOptions *o, const OracleTime *t)
{
    if ((t->time * 1.0) < o->stat_erupt) return 0;
    if ((t->time * 1.0) > o->end_erupt) return 0;
    return 1;
}

/* ------------------------------------------------------------------ */
/* update_pos, update_pos.cc:34-168                                     */
/* ------------------------------------------------------------------ */
static void update_pos(const PlumeOptions *o, PlumeSoA *s, size_t n,
                       const OracleTime *t)
{
    const int D = o->dim;
    double dt = t->dtime;
    int erupt = iferupt(o, t);
    for (size_t i = 0; i < n; i++) {
        uint8_t bc = s->bc_type[i];
        if (is_real(bc)) {
            double v[3];
            vel(s, i, D, o->lans, v);
            s->x[i] = s->x[i] + dt * v[0];
            if (D == 3) {
                s->y[i] = s->y[i] + dt * v[1];
                s->z[i] = s->z[i] + dt * v[2];
            }
        } else if (bc == 0 && erupt) {
            double v[3];
            vel(s, i, D, 0, v);
            s->x[i] = s->x[i] + dt * v[0];
            if (D == 3) {
                s->y[i] = s->y[i] + dt * v[1];
                s->z[i] = s->z[i] + dt * v[2];
                if (s->z[i] >= o->vent_z) {
                    s->bc_type[i] = 100;       /* erupt_turn_real         */
                    s->h[i] = 1.0 * o->sml_phase2; /* put_smlen           */
                    s->involved[i] = 2;        /* set_involved_flag       */
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* update_particles_in_bucket, update_pos.cc:171-463 (serial case)      */
/* Returns the number of deleted particles in *lost_out.                */
/* ------------------------------------------------------------------ */
static void compact(PlumeSoA *s, size_t *n, const char *del);

static int rebucket(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                    size_t *n, const long *old_bucket, size_t *lost_out)
{
    size_t nn = *n, lost = 0;
    char *del = (char *)calloc(nn ? nn : 1, 1);
    int err = PLUME_OK;
    for (size_t i = 0; i < nn; i++) {
        uint8_t bc = s->bc_type[i];
        if (!(is_real(bc) || bc == 0)) continue;
        long ob = old_bucket[i];
        uint8_t of = bucket_flags(g, ob);
        if (of & PLUME_BUCKET_INACTIVE) continue;
        double pos[3] = { s->x[i], s->y[i], s->z[i] };
        if (is_real(bc) && (of & PLUME_BUCKET_MIXED) && g->face_index) {
            /* Bucket::determine_escape, bucket.cc:435-452 */
            const int8_t *fi = g->face_index + 6 * ob;
            int los = 0;
            for (int a = 0; a < 3; a++) {
                if (fi[2 * a] == -1) {
                    if ((pos[a] - g->domain_lo[a]) < -OR_TINY) los = 1;
                } else if (fi[2 * a + 1] == 1) {
                    if ((pos[a] - g->domain_hi[a]) > OR_TINY) los = 1;
                }
            }
            if (los) { del[i] = 1; lost++; continue; }
        }
        long nb_ = bucket_of(g, pos[0], pos[1], pos[2]);
        if (nb_ < 0) { err = PLUME_E_OUTSIDE_GRID; break; }
        if (nb_ != ob && (bucket_flags(g, nb_) & PLUME_BUCKET_ABSORBING)) {
            del[i] = 1;
            lost++;
        }
    }
    if (!err) compact(s, n, del);
    free(del);
    *lost_out = lost;
    return err;
}

#define SOA_D(f) if (s->f) s->f[w] = s->f[r];
static void compact(PlumeSoA *s, size_t *n, const char *del)
{
    size_t w = 0;
    for (size_t r = 0; r < *n; r++) {
        if (del[r]) continue;
        if (w != r) {
            SOA_D(key) SOA_D(x) SOA_D(y) SOA_D(z) SOA_D(vx) SOA_D(vy) SOA_D(vz)
            SOA_D(vsx) SOA_D(vsy) SOA_D(vsz) SOA_D(mass) SOA_D(h) SOA_D(rho)
            SOA_D(e) SOA_D(p) SOA_D(Y) SOA_D(gamma) SOA_D(c) SOA_D(T) SOA_D(cp)
            SOA_D(phase) SOA_D(bc_type) SOA_D(involved)
        }
        w++;
    }
    *n = w;
}
#undef SOA_D

/* ------------------------------------------------------------------ */
/* wall boundary, apply_bcond (bcond.cc:24-249) with BC_FOR_KX 1        */
/* ------------------------------------------------------------------ */
typedef struct Images {
    const uint64_t *key;   /* wall ghost of each image */
    const double   *xyz;   /* image point (3 per image) */
    size_t          n;
} Images;

static int cmp_u64pair(const void *a, const void *b)
{
    const uint64_t *x = (const uint64_t *)a, *y = (const uint64_t *)b;
    return (x[0] > y[0]) - (x[0] < y[0]);
}

/* For every image: the Shepard-normalised SPH averages of rho, v, e (and Y,
 * whose sum the reference accumulates over the neighbour buckets only) of
 * the real and pressure-ghost particles (contr_image, particle.h:562-565)
 * inside CUTOFF2 h_j of the image, over the image's bucket then its 26
 * neighbours in x-major order; the velocity reflected in the wall
 * (reflect, sph_lib.cc:76-83) along the ghost-to-image direction; written
 * to the ghost with its EOS. */
static int apply_bcond(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s, size_t n, const Images *im)
{
    if (!im || im->n == 0) return PLUME_OK;
    long nbk = (long)g->nb[0] * g->nb[1] * g->nb[2];
    long *bk = (long *)malloc(sizeof(long) * (n ? n : 1));
    size_t *bstart = (size_t *)calloc((size_t)nbk + 1, sizeof(size_t));
    int32_t *bidx = (int32_t *)malloc(sizeof(int32_t) * (n ? n : 1));
    uint64_t *kr = (uint64_t *)malloc(sizeof(uint64_t) * 2 * (n ? n : 1));
    if (!bk || !bstart || !bidx || !kr) { free(bk); free(bstart); free(bidx); free(kr); return PLUME_E_INVALID; }
    for (size_t i = 0; i < n; i++) {
        bk[i] = bucket_of(g, s->x[i], s->y[i], s->z[i]);
        if (bk[i] >= 0) bstart[bk[i] + 1]++;
        kr[2 * i] = s->key[i];
        kr[2 * i + 1] = i;
    }
    for (long b = 0; b < nbk; b++) bstart[b + 1] += bstart[b];
    {
        size_t *fill = (size_t *)malloc(sizeof(size_t) * (size_t)(nbk ? nbk : 1));
        memcpy(fill, bstart, sizeof(size_t) * (size_t)nbk);
        for (size_t i = 0; i < n; i++)
            if (bk[i] >= 0) bidx[fill[bk[i]]++] = (int32_t)i;
        free(fill);
    }
    qsort(kr, n, 2 * sizeof(uint64_t), cmp_u64pair);
    int nbx = g->nb[0], nby = g->nb[1], nbz = g->nb[2];
    int rc = PLUME_OK;
    for (size_t q = 0; q < im->n; q++) {
        uint64_t want[2] = { im->key[q], 0 };
        uint64_t *hit = (uint64_t *)bsearch(want, kr, n, 2 * sizeof(uint64_t), cmp_u64pair);
        if (!hit) continue;  /* ghost deleted */
        size_t gi = (size_t)hit[1];
        const double *refc = im->xyz + 3 * q;
        double normal[3], d = 0;
        const double pc[3] = { s->x[gi], s->y[gi], s->z[gi] };
        for (int a = 0; a < 3; a++) { normal[a] = refc[a] - pc[a]; d += normal[a] * normal[a]; }
        for (int a = 0; a < 3; a++) normal[a] /= sqrt(d);
        long b = bucket_of(g, refc[0], refc[1], refc[2]);
        if (b < 0) { rc = PLUME_E_OUTSIDE_GRID; break; }
        double uvec[5] = { 0, 0, 0, 0, 0 }, wnorm = 0, ks = 0;
        int bx = (int)(b % nbx), by = (int)((b / nbx) % nby), bz = (int)(b / ((long)nbx * nby));
        for (int pass = 0; pass < 2; pass++)
            for (int dx = -1; dx <= 1; dx++)
                for (int dy = -1; dy <= 1; dy++)
                    for (int dz = -1; dz <= 1; dz++) {
                        int own = !dx && !dy && !dz;
                        if (own != (pass == 0)) continue;   /* own bucket first */
                        int cx = bx + dx, cy = by + dy, cz = bz + dz;
                        if (cx < 0 || cx >= nbx || cy < 0 || cy >= nby || cz < 0 || cz >= nbz) continue;
                        long nb_ = ((long)cz * nby + cy) * nbx + cx;
                        for (size_t r = bstart[nb_]; r < bstart[nb_ + 1]; r++) {
                            size_t j = (size_t)bidx[r];
                            uint8_t bc = s->bc_type[j];
                            if (!(bc == 100 || bc == 99 || bc == 1)) continue;
                            double h = s->h[j];
                            double ds[3] = { refc[0] - s->x[j], refc[1] - s->y[j], refc[2] - s->z[j] };
                            if (!in_support(ds, o->cutoff2 * h, 3)) continue;
                            double sv[3] = { ds[0] / h, ds[1] / h, ds[2] / h };
                            double w = weight_gauss(sv, h, 3);
                            double mj = s->mass[j], rj = s->rho[j];
                            uvec[0] += mj * w;
                            uvec[1] += mj * w * s->vx[j] / rj;
                            uvec[2] += mj * w * s->vy[j] / rj;
                            uvec[3] += mj * w * s->vz[j] / rj;
                            uvec[4] += mj * w * s->e[j] / rj;
                            if (!own) ks += mj * w * s->Y[j] / rj;
                            wnorm += mj * w / rj;
                        }
                    }
        if (wnorm > 0.) {
            for (int a = 0; a < 5; a++) uvec[a] /= wnorm;
            ks = ks / wnorm;
        } else {
            uvec[0] = 1.;
            for (int a = 1; a < 5; a++) uvec[a] = 0.;
            ks = 0.0;
        }
        double vdotn = uvec[1] * normal[0] + uvec[2] * normal[1] + uvec[3] * normal[2];
        double vr[3];
        for (int a = 0; a < 3; a++) vr[a] = uvec[1 + a] - 2 * vdotn * normal[a];
        s->rho[gi] = uvec[0];
        s->vx[gi] = vr[0]; s->vy[gi] = vr[1]; s->vz[gi] = vr[2];
        s->e[gi] = uvec[4];
        s->Y[gi] = ks;
        eos(o, s, gi);
    }
    free(bk); free(bstart); free(bidx); free(kr);
    return rc;
}

/* ------------------------------------------------------------------ */
/* eruption inlet, add_new_erupt (setup_erupt.cc:389-673)               */
/* ------------------------------------------------------------------ */
typedef struct Inlet {
    const double *xy, *vel;     /* columns */
    uint64_t     *count;        /* particles added per column so far */
    size_t        ncol, cap;    /* cap: rows the particle arrays hold */
    double bot, spacing, mass, h, rho, e, p, gamma, c, Y;
    uint64_t key_base;
} Inlet;

/* Per column, the particles the inflow made room for since the previous
 * step, with the vent state of the Particle constructor (particle.cc:
 * 210-316); key of a column's k-th particle: key_base + k ncol + column. */
static int add_new_erupt(const PlumeOptions *o, PlumeSoA *s, size_t *n, const OracleTime *t,
                         const Inlet *in)
{
    double dt = t->dtime;
    double t_total = t->time - dt;
    for (size_t col = 0; col < in->ncol; col++) {
        double vel = in->vel[col];
        double t_each = in->spacing / vel;
        double t_add = fmod(t_total, t_each) + dt;
        int nn = (int)floor(t_add / t_each);
        t_add = t_add - nn * t_each;
        for (int i = 0; i < nn; i++) {
            if (*n >= in->cap) return PLUME_E_CAPACITY;
            size_t r = (*n)++;
            s->key[r] = in->key_base + in->count[col]++ * (uint64_t)in->ncol + col;
            s->x[r] = in->xy[2 * col];
            s->y[r] = in->xy[2 * col + 1];
            s->z[r] = in->bot + (t_add + i * t_each) * vel;
            s->vx[r] = 0; s->vy[r] = 0; s->vz[r] = vel;
            if (s->vsx) { s->vsx[r] = 0; s->vsy[r] = 0; s->vsz[r] = 0; }
            s->mass[r] = in->mass;
            s->h[r] = in->h;
            s->rho[r] = in->rho;
            s->e[r] = in->e;
            s->Y[r] = in->Y;
            s->phase[r] = 2;
            s->bc_type[r] = 0;
            s->involved[r] = 0;
            s->cp[r] = 0.;
            eos(o, s, r);
            s->p[r] = in->p;
            s->c[r] = in->c;
            s->gamma[r] = in->gamma;
        }
    }
    return PLUME_OK;
}

static int alloc_work(Work *w, size_t n)
{
    size_t m = n ? n : 1;
    w->nv[0] = (double *)malloc(sizeof(double) * m);
    w->nv[1] = (double *)malloc(sizeof(double) * m);
    w->nv[2] = (double *)malloc(sizeof(double) * m);
    w->ne = (double *)malloc(sizeof(double) * m);
    w->nrho = (double *)malloc(sizeof(double) * m);
    w->nY = (double *)malloc(sizeof(double) * m);
    w->nE = (double *)malloc(sizeof(double) * m);
    return (w->nv[0] && w->nv[1] && w->nv[2] && w->ne && w->nrho && w->nY && w->nE)
               ? PLUME_OK : PLUME_E_INVALID;
}
static void free_work(Work *w)
{
    free(w->nv[0]); free(w->nv[1]); free(w->nv[2]);
    free(w->ne); free(w->nrho); free(w->nY); free(w->nE);
}

static int check_opts(const PlumeOptions *o, const PlumeGrid *g, const PlumeSoA *s)
{
    if (!o || !s) return PLUME_E_INVALID;
    if (o->dim != 1 && o->dim != 3) return PLUME_E_INVALID;
    if (o->dim == 3 && (!g || !s->y || !s->z || !s->vy || !s->vz)) return PLUME_E_INVALID;
    return PLUME_OK;
}

static int nthreads_of(int nthreads)
{
#ifdef _OPENMP
    return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
    return 1;
#endif
}

int oracle_adaptive(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                    size_t n, int nthreads)
{
    int rc = check_opts(o, g, s);
    if (rc) return rc;
    nthreads = nthreads_of(nthreads);
    Lists L = { 0 };
    if (o->dim == 3) {
        rc = build_lists_3d(o, g, s, n, (size_t)-1, &L, nthreads);
        if (rc) return rc;
    }
    rc = adaptive_pass(o, s, n, &L, nthreads, (size_t)-1);
    lists_free(&L);
    return rc;
}

/* One step of the hot loop: 3D main.cc:217-471, 1D main.cc:676-750. */
typedef struct GradOut {
    double *grad;
    uint64_t *key;
    size_t cap, n;
} GradOut;
static int steps_impl(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                      size_t *n, OracleTime *t, int nsteps, double *dt_log,
                      int nthreads, const Images *im, const Inlet *inl, GradOut *go);

int oracle_steps(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                 size_t *n, OracleTime *t, int nsteps, double *dt_log,
                 int nthreads)
{
    return steps_impl(o, g, s, n, t, nsteps, dt_log, nthreads, NULL, NULL, NULL);
}

/* oracle_steps plus the GSPH gradients of the last step (n_grad rows with
 * their keys; n_grad = 0 when the step computed none) */
int oracle_steps_grad(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                      size_t *n, OracleTime *t, int nsteps, double *dt_log, int nthreads,
                      double *grad, uint64_t *grad_key, size_t cap, size_t *n_grad)
{
    GradOut go = { grad, grad_key, cap, 0 };
    int rc = steps_impl(o, g, s, n, t, nsteps, dt_log, nthreads, NULL, NULL, &go);
    *n_grad = go.n;
    return rc;
}

int oracle_steps_bc(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                    size_t *n, OracleTime *t, int nsteps, double *dt_log,
                    int nthreads, const uint64_t *img_key, const double *img_xyz,
                    size_t nimg)
{
    Images im = { img_key, img_xyz, nimg };
    return steps_impl(o, g, s, n, t, nsteps, dt_log, nthreads, &im, NULL, NULL);
}

int oracle_steps_inlet(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                       size_t *n, size_t cap, OracleTime *t, int nsteps, double *dt_log,
                       int nthreads, const uint64_t *img_key, const double *img_xyz,
                       size_t nimg, const double *col_xy, const double *col_vel,
                       uint64_t *col_count, size_t ncol, const double *par,
                       uint64_t key_base)
{
    Images im = { img_key, img_xyz, nimg };
    Inlet in = { col_xy, col_vel, col_count, ncol, cap, par[0], par[1], par[2], par[3], par[4],
                 par[5], par[6], par[7], par[8], par[9], key_base };
    return steps_impl(o, g, s, n, t, nsteps, dt_log, nthreads, &im, &in, NULL);
}

int oracle_apply_bcond(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s, size_t n,
                       const uint64_t *img_key, const double *img_xyz, size_t nimg)
{
    Images im = { img_key, img_xyz, nimg };
    return apply_bcond(o, g, s, n, &im);
}

static int steps_impl(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s,
                      size_t *n, OracleTime *t, int nsteps, double *dt_log,
                      int nthreads, const Images *im, const Inlet *inl, GradOut *go)
{
    int rc = check_opts(o, g, s);
    if (rc) return rc;
    nthreads = nthreads_of(nthreads);
    const int D = o->dim;
    for (int st = 0; st < nsteps; st++) {
        size_t nn = *n;
        double dt;
        rc = timestep(o, s, nn, &dt);
        if (rc) return rc;
        incrtime(o, t, &dt);
        if (dt_log) dt_log[st] = dt;
        Lists L = { 0 };
        long *oldb = NULL;
        const int gsph = o->method != PLUME_METHOD_SPH;  /* GSPH or its random choice variant */
        const int recon = gsph && o->gsph_recon != PLUME_RECON_ZEROTH;
        const int need_grad = gsph && (o->gsph_gradients || recon);
        if (D == 3) {
            rc = build_lists_3d_for(o, g, s, nn, (size_t)-1, &L, nthreads, need_grad, NULL);
            if (rc) return rc;
            oldb = (long *)malloc(sizeof(long) * (nn ? nn : 1));
            for (size_t i = 0; i < nn; i++) oldb[i] = bucket_of(g, s->x[i], s->y[i], s->z[i]);
        }
        Work w;
        if (alloc_work(&w, nn)) { lists_free(&L); free(oldb); return PLUME_E_INVALID; }
        int interval = o->sml_interval > 0 ? o->sml_interval : 1;
        if (o->adaptive_sml && (t->step % interval) == 0)
            rc = adaptive_pass(o, s, nn, &L, nthreads, (size_t)-1);
        double *grad = NULL;
        if (!rc && need_grad) {
            /* calc_gradients after adaptive_sml (main.cc:341-343, 697-699) */
            grad = (double *)malloc(sizeof(double) * (nn ? nn : 1) * (size_t)((D + 2) * D));
            if (!grad) rc = PLUME_E_INVALID;
            else gsph_gradients(o, s, nn, &L, grad, nthreads);
        }
        if (!rc) {
            if (gsph) rc = gsph_momentum_pass(o, s, nn, &L, t->dtime, recon ? grad : NULL, &w, nthreads, t->step);
            else rc = momentum_pass(o, s, nn, &L, t->dtime, &w, nthreads);
        }
        if (!rc && go && st == nsteps - 1) {
            go->n = grad ? nn : 0;
            if (grad && nn <= go->cap) {
                memcpy(go->grad, grad, sizeof(double) * nn * (size_t)((D + 2) * D));
                memcpy(go->key, s->key, sizeof(uint64_t) * nn);
            }
        }
        free(grad);
        if (!rc) rc = density_pass(o, s, nn, &L, &w, nthreads);
        if (!rc && o->lans) rc = velocity_pass(o, s, nn, &L, nthreads);
        free_work(&w);
        lists_free(&L);
        if (rc) { free(oldb); return rc; }
        update_pos(o, s, nn, t);
        if (D == 3) {
            size_t lost = 0;
            rc = rebucket(o, g, s, n, oldb, &lost);
            free(oldb);
            if (rc) return rc;
            /* main.cc:416-417 */
            if (inl && inl->ncol && iferupt(o, t)) {
                rc = add_new_erupt(o, s, n, t, inl);
                if (rc) return rc;
            }
            /* main.cc:468, after the inlet and before the output */
            rc = apply_bcond(o, g, s, *n, im);
            if (rc) return rc;
        }
        ifoutput(o, t);
    }
    return PLUME_OK;
}

/* ------------------------------------------------------------------ */
/* domain growth: scan_outside_layer (scan_outside_layer.cc:37-121) and */
/* adapt_domain (adapt_domain.cc:41-194)                                */
/* ------------------------------------------------------------------ */
#define OR_UNDERGROUND 1
#define OR_PRESS_BC    2
#define OR_MIXED       3
#define OR_OVERGROUND  4

/* bucket_type as the harness builds it from the flags: explicit
 * UNDERGROUND / PRESS_BC flags, else an absorbing bucket is below (both z
 * faces -1) or beside the ground */
static int bucket_type_of(const PlumeGrid *g, long b, int explicit_types)
{
    uint8_t f = bucket_flags(g, b);
    if (f & PLUME_BUCKET_MIXED) return OR_MIXED;
    if (f & PLUME_BUCKET_UNDERGROUND) return OR_UNDERGROUND;
    if (f & PLUME_BUCKET_PRESS_BC) return OR_PRESS_BC;
    if ((f & PLUME_BUCKET_ABSORBING) && !explicit_types) {
        const int8_t *fi = g->face_index ? g->face_index + 6 * b : NULL;
        return (fi && fi[4] == -1 && fi[5] == -1) ? OR_UNDERGROUND : OR_PRESS_BC;
    }
    return OR_OVERGROUND;
}

static int explicit_bucket_types(const PlumeGrid *g, long nbk)
{
    for (long b = 0; b < nbk && g->flags; b++)
        if (g->flags[b] & (PLUME_BUCKET_UNDERGROUND | PLUME_BUCKET_PRESS_BC)) return 1;
    return 0;
}

/* the in-grid neighbours of bucket b (26 at most) */
static int bucket_neighbours(const PlumeGrid *g, long b, long *out)
{
    int nx = g->nb[0], ny = g->nb[1], nz = g->nb[2], k = 0;
    int bx = (int)(b % nx), by = (int)((b / nx) % ny), bz = (int)(b / ((long)nx * ny));
    for (int dx = -1; dx <= 1; dx++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dz = -1; dz <= 1; dz++) {
                if (!dx && !dy && !dz) continue;
                int cx = bx + dx, cy = by + dy, cz = bz + dz;
                if (cx < 0 || cx >= nx || cy < 0 || cy >= ny || cz < 0 || cz >= nz) continue;
                out[k++] = ((long)cz * ny + cy) * nx + cx;
            }
    return k;
}

int oracle_scan_outside_layer(const PlumeOptions *o, const PlumeGrid *g, const PlumeSoA *s, size_t n,
                              uint8_t *binv, int *adapt)
{
    if (o->dim != 3 || !binv || !adapt) return PLUME_E_INVALID;
    long nbk = (long)g->nb[0] * g->nb[1] * g->nb[2];
    size_t *cnt = (size_t *)calloc((size_t)nbk, sizeof(size_t));
    char *inv = (char *)calloc((size_t)nbk, 1);
    for (size_t i = 0; i < n; i++) {
        long b = bucket_of(g, s->x[i], s->y[i], s->z[i]);
        if (b < 0) { free(cnt); free(inv); return PLUME_E_OUTSIDE_GRID; }
        cnt[b]++;
        if (s->involved[i] == 2) inv[b] = 1;
    }
    int ex = explicit_bucket_types(g, nbk);
    int a = 0;
    long nbr[26];
    for (long b = 0; b < nbk; b++) {
        if (binv[b] != 1 || !inv[b]) continue;
        binv[b] = 3; /* set_has_involved(HAS_BOTH): bit 1 on */
        int k = bucket_neighbours(g, b, nbr);
        for (int q = 0; q < k; q++) {
            long nb = nbr[q];
            if (cnt[nb] && binv[nb] == 0 && bucket_type_of(g, nb, ex) != OR_UNDERGROUND) {
                a++;
                break;
            }
        }
    }
    *adapt = a;
    free(cnt);
    free(inv);
    return PLUME_OK;
}

/* flags (nbk, in/out): PLUME_BUCKET_ABSORBING leaves the converted buckets */
int oracle_adapt_domain(const PlumeOptions *o, const PlumeGrid *g, PlumeSoA *s, size_t n,
                        uint8_t *binv, uint8_t *flags)
{
    if (o->dim != 3 || !binv) return PLUME_E_INVALID;
    long nbk = (long)g->nb[0] * g->nb[1] * g->nb[2];
    size_t *cnt = (size_t *)calloc((size_t)nbk, sizeof(size_t));
    char *mark = (char *)calloc((size_t)nbk, 1);
    long *bk = (long *)malloc(sizeof(long) * (n ? n : 1));
    for (size_t i = 0; i < n; i++) {
        bk[i] = bucket_of(g, s->x[i], s->y[i], s->z[i]);
        if (bk[i] < 0) { free(cnt); free(mark); free(bk); return PLUME_E_OUTSIDE_GRID; }
        cnt[bk[i]]++;
    }
    int ex = explicit_bucket_types(g, nbk);
    long nbr[26];
    for (long b = 0; b < nbk; b++) {
        int t = bucket_type_of(g, b, ex);
        if (binv[b] != 0 || !cnt[b] || t == OR_UNDERGROUND || t == OR_PRESS_BC) continue;
        int k = bucket_neighbours(g, b, nbr);
        for (int q = 0; q < k; q++)
            if (binv[nbr[q]] & 2) { mark[b] = 1; break; }
    }
    for (long b = 0; b < nbk; b++)
        if (mark[b]) {
            binv[b] = 1; /* set_has_involved(false), set_has_potential_involved(true) */
            if (flags) flags[b] &= (uint8_t)~PLUME_BUCKET_ABSORBING;
        }
    for (size_t i = 0; i < n; i++) {
        long b = bk[i];
        if (!mark[b]) continue;
        int t = bucket_type_of(g, b, ex);
        const int8_t *fi = g->face_index ? g->face_index + 6 * b : NULL;
        int turn;
        if (t == OR_MIXED && fi && fi[4] == -1) {
            turn = s->bc_type[i] == PLUME_BC_PRESSURE; /* on-ground MIXED: its pressure ghosts */
        } else if (t == OR_MIXED) {
            /* other MIXED: particles inside the domain (Bucket::determine_escape) */
            double pos[3] = { s->x[i], s->y[i], s->z[i] };
            int esc = 0;
            for (int a = 0; a < 3 && fi; a++) {
                if (fi[2 * a] == -1) {
                    if ((pos[a] - g->domain_lo[a]) < -OR_TINY) esc = 1;
                } else if (fi[2 * a + 1] == 1) {
                    if ((pos[a] - g->domain_hi[a]) > OR_TINY) esc = 1;
                }
            }
            turn = !esc;
        } else {
            turn = 1; /* OVERGROUND: every particle */
        }
        if (turn) {
            s->bc_type[i] = PLUME_BC_REAL;
            s->involved[i] = 1;
        }
    }
    free(cnt);
    free(mark);
    free(bk);
    return PLUME_OK;
}

static int cmp_u64(const void *a, const void *b)
{
    uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

static int pairs_impl(const PlumeOptions *o, const PlumeGrid *g, const PlumeSoA *s,
                      size_t n, int mode, const char *tmask, uint64_t *key_i, uint64_t *key_j,
                      size_t cap, size_t *npairs)
{
    int rc = check_opts(o, g, s);
    if (rc) return rc;
    const int D = o->dim;
    Lists L = { 0 };
    if (D == 3) {
        rc = build_lists_3d_for(o, g, s, n, (size_t)-1, &L, nthreads_of(0), 0, tmask);
        if (rc) return rc;
    }
    size_t c = 0;
    for (size_t i = 0; i < n; i++) {
        if (!need_neigh(s->bc_type[i])) continue;
        if (tmask && !tmask[i]) continue;
        double xi[3];
        coords(s, i, D, xi);
        double hi = s->h[i];
        FOR_LIST((&L), D, n, i, j, {
            int take = 1;
            if (mode == 1) {
                double xj[3], dx[3], si[3];
                coords(s, j, D, xj);
                double h = 0.5 * (hi + s->h[j]);
                for (int k = 0; k < D; k++) { dx[k] = xi[k] - xj[k]; si[k] = dx[k] / h; }
                take = (j != i) && in_support(dx, o->cutoff2 * hi, D) &&
                       kw(o->kernel, si, h, D) != 0.0;
            }
            if (take) {
                if (c < cap && key_i && key_j) { key_i[c] = s->key[i]; key_j[c] = s->key[j]; }
                c++;
            }
        });
    }
    lists_free(&L);
    *npairs = c;
    return PLUME_OK;
}

int oracle_pairs(const PlumeOptions *o, const PlumeGrid *g, const PlumeSoA *s,
                 size_t n, int mode, uint64_t *key_i, uint64_t *key_j,
                 size_t cap, size_t *npairs)
{
    return pairs_impl(o, g, s, n, mode, NULL, key_i, key_j, cap, npairs);
}

/* oracle_pairs for the need_neigh particles whose keys are in keys[0..nkeys) */
int oracle_pairs_of(const PlumeOptions *o, const PlumeGrid *g, const PlumeSoA *s,
                    size_t n, int mode, const uint64_t *keys, size_t nkeys,
                    uint64_t *key_i, uint64_t *key_j, size_t cap, size_t *npairs)
{
    uint64_t *sk = (uint64_t *)malloc(sizeof(uint64_t) * (nkeys ? nkeys : 1));
    char *tmask = (char *)calloc(n ? n : 1, 1);
    if (!sk || !tmask) { free(sk); free(tmask); return PLUME_E_INVALID; }
    if (nkeys) memcpy(sk, keys, sizeof(uint64_t) * nkeys);
    qsort(sk, nkeys, sizeof(uint64_t), cmp_u64);
    for (size_t i = 0; i < n; i++)
        tmask[i] = nkeys && bsearch(&s->key[i], sk, nkeys, sizeof(uint64_t), cmp_u64) != NULL;
    int rc = pairs_impl(o, g, s, n, mode, tmask, key_i, key_j, cap, npairs);
    free(sk);
    free(tmask);
    return rc;
}

static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

double oracle_sample_step_seconds(const PlumeOptions *o, const PlumeGrid *g,
                                  const PlumeSoA *s0, size_t n, size_t ntarget,
                                  int nthreads)
{
    if (check_opts(o, g, s0) || o->dim != 3) return -1.0;
    nthreads = nthreads_of(nthreads);
    /* private copy of the state so the caller's arrays stay untouched */
    PlumeSoA s = { 0 };
    double *dbuf = (double *)malloc(sizeof(double) * 20 * (n ? n : 1));
    uint8_t *bbuf = (uint8_t *)malloc(3 * (n ? n : 1));
    uint64_t *kbuf = (uint64_t *)malloc(sizeof(uint64_t) * (n ? n : 1));
    if (!dbuf || !bbuf || !kbuf) { free(dbuf); free(bbuf); free(kbuf); return -1.0; }
    double *const src[20] = { s0->x, s0->y, s0->z, s0->vx, s0->vy, s0->vz, s0->vsx,
                              s0->vsy, s0->vsz, s0->mass, s0->h, s0->rho, s0->e, s0->p,
                              s0->Y, s0->gamma, s0->c, s0->T, s0->cp, NULL };
    double **dst[19] = { &s.x, &s.y, &s.z, &s.vx, &s.vy, &s.vz, &s.vsx, &s.vsy, &s.vsz,
                         &s.mass, &s.h, &s.rho, &s.e, &s.p, &s.Y, &s.gamma, &s.c, &s.T, &s.cp };
    for (int f = 0; f < 19; f++) {
        *dst[f] = dbuf + (size_t)f * n;
        memcpy(*dst[f], src[f], sizeof(double) * n);
    }
    s.phase = bbuf; s.bc_type = bbuf + n; s.involved = bbuf + 2 * n;
    memcpy(s.phase, s0->phase, n);
    memcpy(s.bc_type, s0->bc_type, n);
    memcpy(s.involved, s0->involved, n);
    s.key = kbuf;
    memcpy(s.key, s0->key, sizeof(uint64_t) * n);

    double t0 = now_s();
    double dt;
    int rc = timestep(o, &s, n, &dt);
    Lists L = { 0 };
    if (!rc) rc = build_lists_3d(o, g, &s, n, ntarget, &L, nthreads);
    Work w;
    if (!rc) rc = alloc_work(&w, n);
    if (!rc) {
        if (o->adaptive_sml) {
            /* adaptive_sml runs every sml_interval steps: charge its share */
            double ta = now_s();
            adaptive_pass(o, &s, n, &L, nthreads, ntarget);
            double share = (now_s() - ta) * (1.0 - 1.0 / (o->sml_interval > 0 ? o->sml_interval : 1));
            t0 += share;
        }
        momentum_pass(o, &s, n, &L, dt, &w, nthreads);
        density_pass(o, &s, n, &L, &w, nthreads);
        if (o->lans) velocity_pass(o, &s, n, &L, nthreads);
        OracleTime tt = { 0, dt, 1e30, 1, 0 };
        update_pos(o, &s, n, &tt);
        free_work(&w);
    }
    double t1 = now_s();
    lists_free(&L);
    free(dbuf); free(bbuf); free(kbuf);
    return rc ? -1.0 : (t1 - t0);
}
