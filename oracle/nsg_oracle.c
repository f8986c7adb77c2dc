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

/* Fixed-dtau Levi-Civita leapfrog over physical dt, nsphere.c:1827-1937: kick, drift
 * in rho, kick, t += dtau rho_mid^2, until t reaches dt, then linear interpolation
 * (alpha = 1 when the last substep added no time).  The force at the start of a
 * substep is the one at the end of the previous (same operands, same value). */
static int lc_fixed_nf(double r_in, double v_in, double ell, double gnum, double dt, int N_taumin,
                       int64_t max_steps, double *r_out, double *v_out, int nf_stop)
{
    const double l2 = ell * ell;
    double rho = sqrt(r_in), v = v_in, t = 0.0;
    double dtau;
    if (r_in > 1.0e-30 && N_taumin > 0)
        dtau = dt / (2.0 * r_in * (double)N_taumin);
    else
        dtau = dt / 100.0;
    int64_t steps = 0;
    for (;;) {
        if (t >= dt) break;
        const double f = acc_lc(rho, gnum, l2);
        const double vh = v + 0.5 * dtau * f;
        const double rn = rho + dtau * (0.5 * rho * vh);
        const double f2 = acc_lc(rn, gnum, l2);
        const double vn = vh + 0.5 * dtau * f2;
        const double rm = 0.5 * (rho + rn);
        const double tn = t + dtau * (rm * rm);
        if (tn >= dt) {
            double alpha;
            if (fabs(tn - t) > 1.0e-30) alpha = (dt - t) / (tn - t);
            else alpha = 1.0;
            const double rf = rho + alpha * (rn - rho);
            const double vf = v + alpha * (vn - v);
            *r_out = rf * rf;
            *v_out = vf;
            return 0;
        }
        rho = rn; v = vn; t = tn;
        steps++;
        if (steps > max_steps || (nf_stop && !(isfinite(rho) && isfinite(t)))) {
            *r_out = rho * rho;
            *v_out = v;
            return 1;
        }
    }
    *r_out = rho * rho;
    *v_out = v;
    return 0;
}

int orc_lc_fixed(double r_in, double v_in, double ell, double gnum, double dt, int N_taumin,
                 int64_t max_steps, double *r_out, double *v_out)
{
    return lc_fixed_nf(r_in, v_in, ell, gnum, dt, N_taumin, max_steps, r_out, v_out, 0);
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
    if (p->lc_fixed) {   /* method 4, nsphere.c:5696-5707 */
        if (ell != 0.0) {
            const double M_enc = ((double)i / (double)n) * p->M;
            r_crit = (ell * ell) * p->lc_alpha / (p->G * M_enc);
        }
        return (r > 1.0e-30 && r < r_crit);
    }
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
        if (use_lc(p, i, n, ri, li) && p->lc_fixed) {
            capped += lc_fixed_nf(ri, vi, li, gnum, p->dt, p->N_taumin, p->max_tau_steps, &rn, &vn,
                                  p->nonfinite_stop);
            lv = 100;
        } else if (use_lc(p, i, n, ri, li)) {
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
    p->lc_fixed = 0;
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- tracking energies: nsphere.c:6384-6450 with the closed-form potential of the
 * reference's tabulated integrals (nsphere.c:4575-4592); same operation order as the
 * device recorder, each operation rounded once (-ffp-contract=off). ---- */
static double orc_cored_m(double x)
{
    const double u = 1.0 + x * x;
    return (atan(x) + x * (x * x - 1.0) / (u * u)) / 8.0;
}

static double orc_cored_mx_over_x(double x)
{
    if (x < 1e-3) {
        const double t = x * x;
        return t * (1.0 / 3.0 - t * (0.6 - t * (6.0 / 7.0)));
    }
    const double u = 1.0 + x * x;
    return (atan(x) + x * (x * x - 1.0) / (u * u)) / 8.0 / x;
}

double orc_psi(int model, double a, double r_trunc, double r_lo, double r_hi, double G, double M, double r)
{
    if (r < r_lo) r = r_lo + 1e-10;
    else if (r_hi > 0.0 && r > r_hi) r = r_hi - 1e-10;
    const double R = r_trunc;
    if (model == 1) {
        double m = 1.0;
        if (R > 0.0) {
            const double s = R / sqrt(R * R + a * a);
            m = s * s * s;
        }
        return G * M / (m * sqrt(r * r + a * a));
    }
    if (model == 2) {
        double m = 1.0;
        if (R > 0.0) {
            const double s = R / (R + a);
            m = s * s;
        }
        return G * M / (m * (r + a));
    }
    const double m = R > 0.0 ? orc_cored_m(R / a) : 0.19634954084936207;
    const double x = r / a, u = 1.0 + x * x;
    return G * M / (a * m) * (orc_cored_mx_over_x(x) + 0.25 / (u * u));
}

void orc_track(int model, double a, double r_trunc, double r_lo, double r_hi, double G, double M,
               int k, int k_clamped, const double *r, const double *vr, const double *ell, double *out)
{
    for (int t = 0; t < k; t++) {
        double rr = r[t];
        const double v = vr[t], l = ell[t];
        if (t >= k - k_clamped) {
            if (rr < 0.0) rr = 0.0000000001;
            if (r_trunc > 0.0 && rr > r_trunc) rr = r_trunc;
        }
        const double w = v * v + (l * l) / (rr * rr);
        out[t] = rr;
        out[k + t] = v;
        out[2 * k + t] = l;
        out[3 * k + t] = orc_psi(model, a, r_trunc, r_lo, r_hi, G, M, rr) - 0.5 * w;
        out[4 * k + t] = v / sqrt(w);
    }
}

/* ---- per-snapshot post-processing (nsphere.c:7060-7990), sequential restatement ----
 * Natural cubic spline with c_i = y''_i / 2 (the cspline form of the reference's
 * interpolation library), coefficients by the Thomas algorithm. */
static int orc_cspline(int64_t m, const double *x, const double *y, double *c)
{
    if (m < 3) return -1;
    double *cp = (double *)malloc((size_t)m * sizeof(double));
    double *dp = (double *)malloc((size_t)m * sizeof(double));
    if (!cp || !dp) { free(cp); free(dp); return -1; }
    c[0] = 0.0;
    c[m - 1] = 0.0;
    for (int64_t i = 1; i <= m - 2; i++) {
        const double h0 = x[i] - x[i - 1], h1 = x[i + 1] - x[i];
        const double diag = 2.0 * (h0 + h1);
        const double rhs = 3.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
        const double den = (i == 1) ? diag : diag - h0 * cp[i - 1];
        cp[i] = h1 / den;
        dp[i] = (i == 1) ? rhs / den : (rhs - h0 * dp[i - 1]) / den;
    }
    c[m - 2] = dp[m - 2];
    for (int64_t i = m - 3; i >= 1; i--) c[i] = dp[i] - cp[i] * c[i + 1];
    free(cp);
    free(dp);
    return 0;
}

/* largest i <= m-2 with x[i] <= v (x strictly increasing, x[0] <= v) */
static int64_t orc_interval(int64_t m, const double *x, double v)
{
    int64_t lo = 0, hi = m - 1;
    while (hi > lo + 1) {
        const int64_t mid = (lo + hi) / 2;
        if (x[mid] > v) hi = mid;
        else lo = mid;
    }
    return lo;
}

static double orc_cspline_eval(int64_t m, const double *x, const double *y, const double *c, double v)
{
    const int64_t i = orc_interval(m, x, v);
    const double h = x[i + 1] - x[i], dx = v - x[i];
    const double b = (y[i + 1] - y[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
    const double d = (c[i + 1] - c[i]) / (3.0 * h);
    return y[i] + dx * (b + dx * (c[i] + dx * d));
}

/* Smoothed density at each sorted radius (nsphere.c:7281-7686 with the causal
 * Gaussian convolution the zero-padded FFT of :2901-3104 computes, summed directly).
 * Returns 0, or -1 when the reference's validation rejects the radii. */
int orc_density(int64_t n, const double *R, double M, double *rho)
{
    const double dM = M / (double)n;
    /* strictly increasing subsequence and its masses (:7297-7329) */
    double *Rf = (double *)malloc((size_t)n * sizeof(double));
    double *Mf = (double *)malloc((size_t)n * sizeof(double));
    int64_t F = 0;
    for (int64_t i = 0; i < n; i++) {
        if (F == 0 || R[i] > Rf[F - 1]) {
            Rf[F] = R[i];
            Mf[F] = (double)(i + 1) * dM;
            F++;
        }
    }
    /* decimation (:7331-7361) */
    int64_t D = (int64_t)ceil((double)n / 100.0);
    if (D > 30000) D = 30000;
    if (D <= 0) D = 1;
    double *Rd = (double *)malloc((size_t)D * sizeof(double));
    double *Md = (double *)malloc((size_t)D * sizeof(double));
    if (F <= D) {
        D = F;
        memcpy(Rd, Rf, (size_t)F * sizeof(double));
        memcpy(Md, Mf, (size_t)F * sizeof(double));
    } else {
        const double step = (double)(F - 1) / (double)(D - 1);
        for (int64_t i = 0; i < D; i++) {
            int64_t idx = (int64_t)round((double)i * step);
            if (idx >= F) idx = F - 1;
            Rd[i] = Rf[idx];
            Md[i] = Mf[idx];
        }
    }
    free(Rf);
    free(Mf);
    if (D < 3 || !(Rd[0] > 0.0) || !(Rd[D - 1] > Rd[0]) || !isfinite(Rd[D - 1])) {
        free(Rd);
        free(Md);
        return -1;
    }
    /* log grid (:7376-7413) */
    const int64_t G = 131072;
    const double min_r = Rd[0], max_r = Rd[D - 1] * 1.04;
    const double lmin = log10(min_r), lmax = log10(max_r);
    const double dlog = (lmax - lmin) / (double)(G - 1);
    double *lg = (double *)malloc((size_t)G * sizeof(double));
    double *rg = (double *)malloc((size_t)G * sizeof(double));
    double *mg = (double *)malloc((size_t)G * sizeof(double));
    double *dg = (double *)malloc((size_t)G * sizeof(double));
    double *sm = (double *)malloc((size_t)G * sizeof(double));
    double *kn = (double *)malloc((size_t)G * sizeof(double));
    double *cg = (double *)malloc((size_t)G * sizeof(double));
    double *cd = (double *)malloc((size_t)D * sizeof(double));
    for (int64_t i = 0; i < G; i++) {
        lg[i] = lmin + (double)i * dlog;
        rg[i] = pow(10.0, lg[i]);
    }
    for (int64_t i = 1; i < G; i++)
        if (rg[i] <= rg[i - 1]) rg[i] = rg[i - 1] + 1e-12;
    for (int64_t i = 1; i < D; i++)
        if (Rd[i] <= Rd[i - 1]) Rd[i] = Rd[i - 1] + 1e-12;
    /* M(r) on the grid (:7415-7494) */
    orc_cspline(D, Rd, Md, cd);
    for (int64_t i = 0; i < G; i++) {
        if (rg[i] < Rd[0]) mg[i] = Md[0];
        else if (rg[i] > Rd[D - 1]) mg[i] = Md[D - 1];
        else mg[i] = orc_cspline_eval(D, Rd, Md, cd, rg[i]);
    }
    /* dM/dr by central differences (:7496-7521) */
    for (int64_t i = 1; i < G - 1; i++) {
        const double dr = rg[i + 1] - rg[i - 1];
        if (dr > 1e-15) dg[i] = (mg[i + 1] - mg[i - 1]) / dr;
        else dg[i] = (i > 1) ? dg[i - 1] : 0.0;
        if (dg[i] < 1e-10) dg[i] = 1e-10;
    }
    dg[0] = dg[1];
    dg[G - 1] = dg[G - 2];
    /* Gaussian smoothing in log r (:7539-7570, :2901-3104) */
    const double sigma = 0.08 * pow((double)n / 10000.0, -0.40);
    const double step = lg[1] - lg[0];
    const double pref = 1.0 / (sigma * sqrt(2.0 * M_PI));
    double norm = 0.0;
    int64_t W = 0;
    for (int64_t m = 0; m < G; m++) {
        const double x = (double)m * step;
        kn[m] = pref * exp(-0.5 * (x / sigma) * (x / sigma));
        norm += kn[m];
        if (kn[m] > 0.0) W = m;
    }
    for (int64_t m = 0; m < G; m++) kn[m] /= norm;
    for (int64_t i = 0; i < G; i++) {
        double s = 0.0;
        const int64_t top = i < W ? i : W;
        for (int64_t m = 0; m <= top; m++) s += kn[m] * dg[i - m];
        sm[i] = s < 1e-10 ? 1e-10 : s;
    }
    /* back to the particles (:7572-7658) */
    orc_cspline(G, rg, sm, cg);
    for (int64_t i = 0; i < n; i++) {
        const double v = R[i];
        if (v <= rg[0]) rho[i] = sm[0];
        else if (v >= rg[G - 1]) rho[i] = sm[G - 1];
        else rho[i] = orc_cspline_eval(G, rg, sm, cg, v);
    }
    free(Rd); free(Md); free(lg); free(rg); free(mg); free(dg); free(sm); free(kn); free(cg); free(cd);
    return 0;
}

/* Knots of the Psi_A interpolation (nsphere.c:7752-7768): (0, R_0, ..., R_{n-1}) with
 * every knot not above its predecessor moved to the predecessor + 1e-5. */
void orc_psi_knots(int64_t n, const double *R, double *knots)
{
    knots[0] = 0.0;
    for (int64_t i = 1; i <= n; i++) {
        knots[i] = R[i - 1];
        if (knots[i] <= knots[i - 1]) knots[i] = knots[i - 1] + 1e-5;
    }
}

/* linear interpolation on strictly increasing knots; NaN outside */
static double orc_linear_eval(int64_t m, const double *x, const double *y, double v)
{
    if (!(v >= x[0] && v <= x[m - 1])) return NAN;
    const int64_t i = orc_interval(m, x, v);
    const double dx = x[i + 1] - x[i];
    return y[i] + (v - x[i]) / dx * (y[i + 1] - y[i]);
}

typedef struct { float rad; int64_t idx; } orc_rad_idx;
static int orc_cmp_rad(const void *a, const void *b)
{
    const orc_rad_idx *p = (const orc_rad_idx *)a, *q = (const orc_rad_idx *)b;
    if (p->rad < q->rad) return -1;
    if (p->rad > q->rad) return 1;
    return (p->idx > q->idx) - (p->idx < q->idx);
}

int orc_post_snapshot(int64_t n, const float *r, const float *v, const float *l, double G, double M,
                      int64_t *s_idx, double *s_r, double *s_v, double *s_l, double *s_psi, double *s_E,
                      double *s_rho, double *u_psi, double *u_E, double *psi0)
{
    const double dM = M / (double)n;
    orc_rad_idx *pa = (orc_rad_idx *)malloc((size_t)n * sizeof(orc_rad_idx));
    for (int64_t i = 0; i < n; i++) {
        pa[i].rad = (r[i] != r[i]) ? 0.0f : r[i];
        pa[i].idx = i;
    }
    qsort(pa, (size_t)n, sizeof(orc_rad_idx), orc_cmp_rad);
    for (int64_t i = 0; i < n; i++) {
        const int64_t o = pa[i].idx;
        s_idx[i] = o;
        s_r[i] = (double)pa[i].rad;
        s_v[i] = (v[o] != v[o]) ? 0.0 : (double)v[o];
        s_l[i] = (double)l[o];
    }
    free(pa);
    int rc = orc_density(n, s_r, M, s_rho);
    /* Psi_A at the sorted radii (:7697-7734) */
    double *psiA = (double *)malloc((size_t)(n + 1) * sizeof(double));
    double *kx = (double *)malloc((size_t)(n + 1) * sizeof(double));
    double *suffix = (double *)malloc((size_t)n * sizeof(double));
    suffix[n - 1] = 1.0 / s_r[n - 1];
    for (int64_t j = n - 2; j >= 0; j--) suffix[j] = suffix[j + 1] + 1.0 / s_r[j];
    double sum = 0.0;
    for (int64_t j = 0; j < n; j++) sum += 1.0 / s_r[j];
    *psi0 = G * dM * sum;
    psiA[0] = *psi0;
    for (int64_t i = 0; i < n; i++) {
        const double outer = (i < n - 1) ? dM * suffix[i + 1] : 0.0;
        psiA[i + 1] = G * (((double)(i + 1) * dM) / s_r[i] + outer);
    }
    orc_psi_knots(n, s_r, kx);
    for (int64_t i = 0; i < n; i++) {
        const double rr = s_r[i];
        s_psi[i] = orc_linear_eval(n + 1, kx, psiA, rr);
        s_E[i] = s_psi[i] - (s_l[i] * s_l[i] / (2.0 * rr * rr)) - 0.5 * s_v[i] * s_v[i];
    }
    for (int64_t i = 0; i < n; i++) {
        const double rr = (double)r[i], vv = (double)v[i], ll = (double)l[i];
        u_psi[i] = orc_linear_eval(n + 1, kx, psiA, rr);
        u_E[i] = u_psi[i] - (ll * ll / (2.0 * rr * rr)) - 0.5 * vv * vv;
    }
    free(psiA);
    free(kx);
    free(suffix);
    return rc;
}
