/*
 * nsg_oracle.c -- CPU oracle for the NSphere per-step shell loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library in
 * nsphere_gb300/csrc is compared against.  Only tests/, the smoke check in
 * __graft_entry__.py and the cpu_baseline leg of bench.py load it; the product
 * path never calls it and has no CPU fallback.
 *
 * It is a plain-C restatement of the reference algorithm (kris-sigurdson/NSphere
 * v0.1.2, src/c/nsphere.c), written for this project.  Every function names the
 * reference lines it follows.  Arithmetic is written in the reference's operation
 * order and the file is compiled with -O2 -fno-fast-math -ffp-contract=off, so each
 * IEEE-754 double operation rounds exactly as the reference's does when the
 * reference is built with the same flags.  The restatement is pinned against the
 * reference's own functions (built from their sources by oracle/build_ref.sh into
 * oracle/_ref) by tests/test_oracle_pin.py and by the fixtures in tests/golden/.
 *
 * Contract differences that are deliberate and documented:
 *   - the radial sort is a total order on (r, id): ties in r are broken by the
 *     particle id, -0.0 equals +0.0, NaN sorts last.  The reference's stable
 *     quadsort (src/c/quadsort.h:300) breaks ties by the previous array order;
 *     both agree whenever the radii are distinct.
 *   - the Levi-Civita tau-step cap is a parameter (reference: 1e8, nsphere.c:2273).
 *
 * Units: G_eff is the reference's (VEL_CONV_SQ * G_CONST) product, M is HALO_MASS.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "nsg_oracle.h"

/* ---------------------------------------------------------------- forces -- */

/* Numerator of the shell-theorem gravity for a particle of 0-based rank i among n:
 * -(G_eff) * (i/n) * M, in the reference's left-to-right order (nsphere.c:513). */
double orc_gnum(int64_t i, int64_t n, double G, double M)
{
    return (-(G) * ((double)i / (double)n)) * M;
}

/* The gravity numerator with a central point mass Mpt, the build's extension for the
 * point-mass configuration (the reference has none): gnum - G Mpt when Mpt != 0. */
double orc_gnum_pm(int64_t i, int64_t n, double G, double M, double Mpt)
{
    double g = orc_gnum(i, n, G, M);
    if (Mpt != 0.0) g = g - G * Mpt;
    return g;
}

/* dv/dt = gravity + centrifugal, nsphere.c:502-515 and :532-535.
 * gravity = gnum / (r*r), centrifugal = (ell*ell) / (r*r*r). */
static inline double acc_leap(double r, double gnum, double l2)
{
    double f = gnum / (r * r);
    double a = l2 / (r * r * r);
    return f + a;
}

/* Levi-Civita force in rho = sqrt(r), nsphere.c:563-575, :596-599, :1777-1787:
 * gnum / (rho*rho) + (ell*ell) / (rho*rho*rho*rho). */
static inline double acc_lc(double rho, double gnum, double l2)
{
    double g = gnum / (rho * rho);
    double a = l2 / (rho * rho * rho * rho);
    return g + a;
}

/* ------------------------------------------------------- adaptive leapfrog -- */

/* Kick-drift-kick over h with N coarse or 2N fine substeps, nsphere.c:1550-1607. */
void orc_micro_leap(double r_in, double v_in, double l2, double gnum, double h,
                    int64_t N, int fine, double *r_out, double *v_out)
{
    double halfKick, midStep;
    if (!fine) {                       /* subSteps == 2N+1 */
        halfKick = h / (2.0 * (double)N);
        midStep = h / (1.0 * (double)N);
    } else {                           /* subSteps == 4N+1 */
        halfKick = h / (4.0 * (double)N);
        midStep = h / (2.0 * (double)N);
    }
    int64_t pairs = fine ? 2 * N : N;  /* (subSteps - 1) / 2 */
    double r = r_in, v = v_in;
    v += halfKick * acc_leap(r, gnum, l2);
    for (int64_t pp = 1; pp <= pairs - 1; pp++) {
        r += midStep * v;
        v += midStep * acc_leap(r, gnum, l2);
    }
    r += midStep * v;
    v += halfKick * acc_leap(r, gnum, l2);
    *r_out = r;
    *v_out = v;
}

/* Adaptive full leapfrog step, nsphere.c:1648-1735.  N = 1, 2, 4, ... <= max_subdiv;
 * accepts when both relative coarse/fine differences are below tolerance.
 * *level receives log2(N) of the accepted level, or -1 when no level converged. */
static void adaptive_leap_nf(double r_in, double v_in, double ell, double gnum, double h,
                             double tol_r, double tol_v, int64_t max_subdiv, int out_type,
                             double *r_out, double *v_out, int *level, int nf_stop)
{
    double l2 = ell * ell;
    double rc = r_in, vc = v_in, rf = r_in, vf = v_in;
    int64_t N = 1;
    int k = 0;
    while (N <= max_subdiv) {
        orc_micro_leap(r_in, v_in, l2, gnum, h, N, 0, &rc, &vc);
        orc_micro_leap(r_in, v_in, l2, gnum, h, N, 1, &rf, &vf);
        double dr = fabs(rf - rc) / (fabs(rf) + 1.0e-30);
        double dv = fabs(vf - vc) / (fabs(vf) + 1.0e-30);
        if (dr < tol_r && dv < tol_v) {
            *level = k;
            goto out;
        }
        /* the build's bounded-work rule (nonfinite_stop): a non-finite pass ends the
         * climb; the reference keeps climbing to max_subdiv */
        if (nf_stop && !(isfinite(rf) && isfinite(vf))) break;
        N *= 2;
        k++;
    }
    *level = -1;
out:
    if (out_type == 0) {
        *r_out = rc; *v_out = vc;
    } else if (out_type == 1) {
        *r_out = rf; *v_out = vf;
    } else {
        *r_out = 4.0 * rf - 3.0 * rc;
        *v_out = 4.0 * vf - 3.0 * vc;
    }
}

/* ------------------------------------------------------------ Levi-Civita -- */

/* subSteps tau-leapfrog substeps over h_tau in (rho, v, t), nsphere.c:1990-2036. */
static void micro_lc(double rho_in, double v_in, double t_in, int64_t subSteps,
                     double h_tau, double gnum, double l2,
                     double *rho_out, double *v_out, double *t_out)
{
    double dtau = h_tau / (double)subSteps;
    double rho = rho_in, v = v_in, t = t_in;
    for (int64_t ss = 0; ss < subSteps; ss++) {
        double f1 = acc_lc(rho, gnum, l2);
        double vh = v + 0.5 * dtau * f1;
        double rn = rho + dtau * (0.5 * rho * vh);
        double f2 = acc_lc(rn, gnum, l2);
        double vn = vh + 0.5 * dtau * f2;
        double rm = 0.5 * (rho + rn);
        t += dtau * (rm * rm);
        rho = rn;
        v = vn;
    }
    *rho_out = rho; *v_out = v; *t_out = t;
}

/* One adaptive tau-step, nsphere.c:2077-2186.  Returns log2(N) accepted, or -1 when
 * the fallback fine pass at 4*(2*N_last)+1 substeps was used. */
static int tau_step_lc(double rho_in, double v_in, double t_in, double h_guess,
                       double tol_r, double tol_v, int64_t max_subdiv, double gnum,
                       double l2, int out_type,
                       double *rho_out, double *v_out, double *t_out, int nf_stop)
{
    int64_t N = 1;
    int k = 0;
    while (N <= max_subdiv) {
        double rC, vC, tC, rF, vF, tF;
        micro_lc(rho_in, v_in, t_in, 2 * N + 1, h_guess, gnum, l2, &rC, &vC, &tC);
        micro_lc(rho_in, v_in, t_in, 4 * N + 1, h_guess, gnum, l2, &rF, &vF, &tF);
        double rsq = rF * rF;
        double drho = fabs(rF - rC) / (fabs(rsq) + 1.0e-30);
        double dv = fabs(vF - vC) / (fabs(vF) + 1.0e-30);
        if (drho < tol_r && dv < tol_v) {
            if (out_type == 0) {
                *rho_out = rC; *v_out = vC; *t_out = tC;
            } else if (out_type == 1) {
                *rho_out = rF; *v_out = vF; *t_out = tF;
            } else {
                double rr = 4.0 * rF - 3.0 * rC;
                double vr = 4.0 * vF - 3.0 * vC;
                double tr = 4.0 * tF - 3.0 * tC;
                if (rr < 0.0) rr = 0.0;
                *rho_out = rr; *v_out = vr; *t_out = tr;
            }
            return k;
        }
        if (nf_stop && !(isfinite(rF) && isfinite(vF))) {   /* bounded-work rule */
            *rho_out = rF; *v_out = vF; *t_out = tF;
            return -1;
        }
        N *= 2;
        k++;
    }
    micro_lc(rho_in, v_in, t_in, 4 * N + 1, h_guess, gnum, l2, rho_out, v_out, t_out);
    return -1;
}

/* Adaptive full Levi-Civita step over physical dt, nsphere.c:2231-2334.
 * *level receives the highest accepted tau-step level (-1 if any tau-step fell
 * back), *ntau the number of tau-steps taken.  Returns 1 when the tau-step cap
 * was hit (the reference's stepMax exit), else 0. */
static int adaptive_lc_nf(double r_in, double v_in, double ell, double gnum, double dt,
                          int N_taumin, double tol_r, double tol_v, int64_t max_subdiv,
                          int out_type, int64_t max_tau_steps,
                          double *r_out, double *v_out, int *level, int64_t *ntau, int nf_stop)
{
    *level = 0;
    *ntau = 0;
    if (r_in < 1.0e-30) {
        *r_out = r_in; *v_out = v_in;
        return 0;
    }
    double l2 = ell * ell;
    double rho = sqrt(r_in);
    double v = v_in;
    double t = 0.0;
    double dtau;
    if (r_in > 1.0e-30 && N_taumin > 0)
        dtau = dt / (2.0 * r_in * (double)N_taumin);
    else
        dtau = dt / 100.0;
    int64_t steps = 0;
    int lvmax = 0;
    for (;;) {
        if (t >= dt) break;
        double rn, vn, tn;
        int lv = tau_step_lc(rho, v, t, dtau, tol_r, tol_v, max_subdiv, gnum, l2,
                             out_type, &rn, &vn, &tn, nf_stop);
        if (lv < 0) lvmax = -1;
        else if (lvmax >= 0 && lv > lvmax) lvmax = lv;
        *ntau = steps + 1;
        if (tn > dt) {
            double alpha = 0.0;
            if (fabs(tn - t) > 1.0e-30) alpha = (dt - t) / (tn - t);
            double rf = rho + alpha * (rn - rho);
            double vf = v + alpha * (vn - v);
            *r_out = rf * rf; *v_out = vf;
            *level = lvmax;
            return 0;
        }
        rho = rn; v = vn; t = tn;
        steps++;
        if (steps > max_tau_steps || (nf_stop && !(isfinite(rho) && isfinite(t)))) {
            *r_out = rho * rho; *v_out = v;
            *level = lvmax;
            return 1;
        }
    }
    *r_out = rho * rho; *v_out = v;
    *level = lvmax;
    return 0;
}

/* The per-particle integrators as the reference runs them (no bounded-work rule). */
void orc_adaptive_leap(double r_in, double v_in, double ell, double gnum, double h,
                       double tol_r, double tol_v, int64_t max_subdiv, int out_type,
                       double *r_out, double *v_out, int *level)
{
    adaptive_leap_nf(r_in, v_in, ell, gnum, h, tol_r, tol_v, max_subdiv, out_type, r_out, v_out, level, 0);
}

int orc_adaptive_lc(double r_in, double v_in, double ell, double gnum, double dt,
                    int N_taumin, double tol_r, double tol_v, int64_t max_subdiv,
                    int out_type, int64_t max_tau_steps,
                    double *r_out, double *v_out, int *level, int64_t *ntau)
{
    return adaptive_lc_nf(r_in, v_in, ell, gnum, dt, N_taumin, tol_r, tol_v, max_subdiv, out_type,
                          max_tau_steps, r_out, v_out, level, ntau, 0);
}

/* ------------------------------------------------------------------- sort -- */

typedef struct { double r; int32_t id; int32_t src; } sort_item;

/* (r, id) total order: -0.0 == +0.0 compare equal and fall to the id; NaN last. */
static int cmp_item(const void *pa, const void *pb)
{
    const sort_item *a = (const sort_item *)pa, *b = (const sort_item *)pb;
    int na = isnan(a->r), nb = isnan(b->r);
    if (na != nb) return na ? 1 : -1;
    if (!na) {
        if (a->r < b->r) return -1;
        if (a->r > b->r) return 1;
    }
    return (a->id > b->id) - (a->id < b->id);
}

/* Stable radial sort of the state, in place (the contract of sort_particles,
 * nsphere.c:8605-8665, with ties on r broken by particle id).  aux may be NULL;
 * when given it is permuted along (the reference's fifth column, mu). */
int orc_sort(int64_t n, double *r, double *vr, double *ell, int32_t *id, double *aux)
{
    if (n <= 0) return 0;
    sort_item *it = (sort_item *)malloc((size_t)n * sizeof(sort_item));
    double *tmp = (double *)malloc((size_t)n * sizeof(double));
    int32_t *tid = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!it || !tmp || !tid) { free(it); free(tmp); free(tid); return -1; }
    for (int64_t k = 0; k < n; k++) { it[k].r = r[k]; it[k].id = id[k]; it[k].src = (int32_t)k; }
    qsort(it, (size_t)n, sizeof(sort_item), cmp_item);
    double *cols[4] = { r, vr, ell, aux };
    for (int c = 0; c < 4; c++) {
        double *col = cols[c];
        if (!col) continue;
        for (int64_t k = 0; k < n; k++) tmp[k] = col[it[k].src];
        memcpy(col, tmp, (size_t)n * sizeof(double));
    }
    for (int64_t k = 0; k < n; k++) tid[k] = id[it[k].src];
    memcpy(id, tid, (size_t)n * sizeof(int32_t));
    free(it); free(tmp); free(tid);
    return 0;
}

/* ------------------------------------------------------------ step bodies -- */

/* r_crit routing of the method-5 body, nsphere.c:5804-5822 (alpha rule), or a
 * fixed radius (lc_rule 1), or never (lc_rule 2).  Returns 1 for Levi-Civita. */
static int use_lc(const orc_params *p, int64_t i, int64_t n, double r, double ell)
{
    if (p->lc_rule == 2) return 0;
    if (p->lc_rule == 1) return (r > 1.0e-30 && r < p->lc_radius);
    double r_crit = 0.0;
    if (fabs(ell) > 1.0e-30) {
        double M_enc;
        if (i == 0) M_enc = 0.1 * (1.0 / (double)n) * p->M;
        else M_enc = ((double)i / (double)n) * p->M;
        double gravPart = p->G * M_enc;
        r_crit = (ell * ell) * p->lc_alpha / gravPart;
    }
    return (r > 1.0e-30 && r < r_crit);
}

/* One method-5 step (nsphere.c:5775-5838): sort, then for each rank route to the
 * adaptive Levi-Civita or adaptive leapfrog integrator.  level[i] (may be NULL)
 * receives the accepted level per sorted position; LC particles get 100 + level
 * (or 99 for a fallback), so tests can tell the two paths apart.  Returns the
 * number of particles that hit the tau-step cap. */
int64_t orc_step_adaptive(const orc_params *p, int64_t n, double *r, double *vr,
                          double *ell, int32_t *id, int8_t *level)
{
    if (orc_sort(n, r, vr, ell, id, NULL) != 0) return -1;
    int64_t capped = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+:capped)
    for (int64_t i = 0; i < n; i++) {
        double ri = r[i], vi = vr[i], li = ell[i];
        double gnum = orc_gnum_pm(i, n, p->G, p->M, p->point_mass);
        double rn, vn;
        int lv;
        if (use_lc(p, i, n, ri, li)) {
            int64_t nt;
            capped += adaptive_lc_nf(ri, vi, li, gnum, p->dt, p->N_taumin, p->tol_r,
                                     p->tol_v, p->max_subdiv, p->out_type,
                                     p->max_tau_steps, &rn, &vn, &lv, &nt, p->nonfinite_stop);
            lv = (lv < 0) ? 99 : 100 + lv;
        } else {
            adaptive_leap_nf(ri, vi, li, gnum, p->dt, p->tol_r, p->tol_v,
                             p->max_subdiv, p->out_type, &rn, &vn, &lv, p->nonfinite_stop);
        }
        r[i] = rn;
        vr[i] = vn;
        if (level) level[i] = (int8_t)lv;
    }
    return capped;
}

/* One fixed-step kick-drift-sort-kick step, nsphere.c:5484-5531 (method 6 on the
 * command line, internal method 2).  The first kick uses the rank of the order the
 * state arrives in, as the reference does. */
void orc_step_kdk(const orc_params *p, int64_t n, double *r, double *vr, double *ell,
                  int32_t *id)
{
    double dt = p->dt;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double a = acc_leap(r[i], orc_gnum_pm(i, n, p->G, p->M, p->point_mass), ell[i] * ell[i]);
        vr[i] = vr[i] + 0.5 * a * dt;
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) r[i] += vr[i] * dt;
    orc_sort(n, r, vr, ell, id, NULL);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double a = acc_leap(r[i], orc_gnum_pm(i, n, p->G, p->M, p->point_mass), ell[i] * ell[i]);
        vr[i] = vr[i] + 0.5 * a * dt;
    }
}

/* Total energy of a state in sorted order, consistent with the rank force law:
 * K = sum 1/2 m (v^2 + ell^2/r^2), W = sum m * gnum_i / r_i with m = M/n.
 * Summed in index order (the device sums in a fixed tree order; tests compare
 * to a relative tolerance). */
void orc_energy(const orc_params *p, int64_t n, const double *r, const double *vr,
                const double *ell, double *K, double *W)
{
    double m = p->M / (double)n;
    double k = 0.0, w = 0.0;
    for (int64_t i = 0; i < n; i++) {
        double ri = r[i];
        k += 0.5 * m * (vr[i] * vr[i] + (ell[i] * ell[i]) / (ri * ri));
        w += m * orc_gnum_pm(i, n, p->G, p->M, p->point_mass) / ri;
    }
    *K = k;
    *W = w;
}

void orc_params_default(orc_params *p)
{
    p->G = 1.0;
    p->M = 1.0;
    p->dt = 5.0e-4;
    p->tol_r = 1.0e-7;
    p->tol_v = 1.0e-7;
    p->max_subdiv = 128;
    p->out_type = 2;
    p->N_taumin = 10;
    p->lc_rule = 0;
    p->lc_alpha = 0.05;
    p->lc_radius = 1.0e-3;
    p->max_tau_steps = 100000000;
    p->point_mass = 0.0;
    p->nonfinite_stop = 1;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
