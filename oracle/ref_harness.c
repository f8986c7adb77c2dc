/*
 * ref_harness.c -- exported wrappers around the reference's own hot-path functions
 * (TEST INFRASTRUCTURE ONLY; used to pin oracle/nsg_oracle.c and as the timed CPU
 * reference of bench.py).
 *
 * Compiled by oracle/build_ref.py together with oracle/_ref/ref_hotpath.c, the
 * reference's functions extracted verbatim from src/c/nsphere.c at build time.
 * The step loops below restate the inline time-loop bodies of main()
 * (nsphere.c:5775-5838 for method 5, nsphere.c:5484-5531 for method 2) around the
 * reference's own sort_particles and integrators; the reference has no callable
 * step function to wrap.
 */
#include "ref_hotpath.c"

/* Mirrors the harness globals: G (G_CONST, with VEL_CONV_SQ = 1) and HALO_MASS. */
void ref_set_units(double G, double M)
{
    ref_G_value = G;
    ref_halo_mass = M;
}

/* "quadsort" (exact, stable) or "quadsort_parallel" (the reference default). */
void ref_set_sort(int parallel)
{
    g_defaultSortAlg = parallel ? "quadsort_parallel" : "quadsort";
}

void ref_adaptive_leap(int i, int npts, double r, double v, double ell, double h,
                       double tol_r, double tol_v, int max_subdiv, int out_type,
                       double *r_out, double *v_out)
{
    doAdaptiveFullLeap(i, npts, r, v, ell, h, tol_r, tol_v, max_subdiv, G_CONST, out_type,
                       r_out, v_out);
}

void ref_adaptive_lc(int i, int npts, double r, double v, double ell, double dt, int N_taumin,
                     double tol_r, double tol_v, int max_subdiv, int out_type,
                     double *r_out, double *v_out)
{
    doAdaptiveFullLeviCivita(i, npts, r, v, ell, dt, N_taumin, tol_r, tol_v, max_subdiv,
                             G_CONST, out_type, r_out, v_out);
}

void ref_lc_fixed(int i, int npts, double r, double v, double ell, double dt, int N_taumin,
                  double *r_out, double *v_out)
{
    doLeviCivitaLeapfrog(i, npts, r, v, ell, dt, N_taumin, G_CONST, r_out, v_out);
}

void ref_micro_leap(int i, int npts, double r, double v, double ell, double h, int N,
                    int subSteps, double *r_out, double *v_out)
{
    doMicroLeapfrog(i, npts, r, v, ell, h, N, subSteps, G_CONST, r_out, v_out);
}

/* sort_particles on the five-column table particles[5][npts] (nsphere.c:8662). */
void ref_sort_particles(double **particles, int npts)
{
    sort_particles(particles, npts);
}

/* One method-5 step as in main() (nsphere.c:5775-5838), with the reference's
 * constants except max_subdiv and the routing rule, which are arguments
 * (lc_rule 0: the r_crit rule of nsphere.c:5804-5822; 1: r < lc_radius). */
void ref_step_method5(double **particles, int npts, double dt, int max_subdiv,
                      int lc_rule, double lc_radius, int *inverse_map)
{
    double velocity_tol = 1.0e-7;
    double radius_tol = 1.0e-7;
    int out_type = 2;
    int N_taumin = 10;
    double alpha_param = 0.05;

    sort_particles(particles, npts);
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < npts; idx++) {
        int orig_id = (int)particles[3][idx];
        inverse_map[orig_id] = idx;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < npts; i++) {
        double r = particles[0][i];
        double v = particles[1][i];
        double ell = particles[2][i];
        double r_crit = 0.0;
        if (lc_rule == 1) {
            r_crit = lc_radius;
        } else if (fabs(ell) > 1.0e-30) {
            double M_enc;
            if (i == 0) M_enc = 0.1 * (1.0 / (double)npts) * HALO_MASS;
            else M_enc = ((double)i / (double)npts) * HALO_MASS;
            double gravPart = (VEL_CONV_SQ * G_CONST) * M_enc;
            r_crit = (ell * ell) * alpha_param / gravPart;
        }
        double r_new, v_new;
        if (r > 1.0e-30 && r < r_crit)
            doAdaptiveFullLeviCivita(i, npts, r, v, ell, dt, N_taumin, radius_tol, velocity_tol,
                                     max_subdiv, G_CONST, out_type, &r_new, &v_new);
        else
            doAdaptiveFullLeap(i, npts, r, v, ell, dt, radius_tol, velocity_tol, max_subdiv,
                               G_CONST, out_type, &r_new, &v_new);
        particles[0][i] = r_new;
        particles[1][i] = v_new;
    }
}

/* One method-4 step (CLI --method 2) as in main() (nsphere.c:5661-5745), with the
 * reference's constants except max_subdiv, the tolerance and N_taumin, which are
 * arguments (the reference: 4096*4096, 1e-8, 1000). */
void ref_step_method4(double **particles, int npts, double dt, int max_subdiv, double tol,
                      int N_taumin, int *inverse_map)
{
    int out_type = 2;
    double alpha_param = 0.05;
    sort_particles(particles, npts);
#pragma omp parallel for schedule(dynamic, 64)
    for (int i = 0; i < npts; i++) {
        double r = particles[0][i];
        double v = particles[1][i];
        double ell = particles[2][i];
        double r_crit = 0.0;
        if (ell != 0.0) {
            double M_enc = ((double)i / (double)npts) * HALO_MASS;
            double gravPart = (VEL_CONV_SQ * G_CONST) * M_enc;
            r_crit = (ell * ell) * (alpha_param) / (gravPart);
        }
        double r_new, v_new;
        if ((r > 1.0e-30) && (r < r_crit))
            doLeviCivitaLeapfrog(i, npts, r, v, ell, dt, N_taumin, G_CONST, &r_new, &v_new);
        else
            doAdaptiveFullLeap(i, npts, r, v, ell, dt, tol, tol, max_subdiv, G_CONST, out_type,
                               &r_new, &v_new);
        particles[0][i] = r_new;
        particles[1][i] = v_new;
    }
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < npts; idx++) {
        int orig_id = (int)particles[3][idx];
        inverse_map[orig_id] = idx;
    }
}

/* One method-2 step (CLI --method 6) as in main() (nsphere.c:5484-5531). */
void ref_step_kdk(double **particles, int npts, double dt, int *inverse_map)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npts; i++) {
        double r = particles[0][i];
        double vrad = particles[1][i];
        double ell = particles[2][i];
        double force = gravitational_force(r, i, npts, G_CONST, HALO_MASS);
        double dvdt = force + effective_angular_force(r, ell);
        particles[1][i] = vrad + 0.5 * dvdt * dt;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npts; i++) {
        double vrad = particles[1][i];
        particles[0][i] += vrad * dt;
    }
    sort_particles(particles, npts);
#pragma omp parallel for schedule(static)
    for (int idx = 0; idx < npts; idx++) {
        int orig_id = (int)particles[3][idx];
        inverse_map[orig_id] = idx;
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < npts; i++) {
        double r = particles[0][i];
        double vrad = particles[1][i];
        double ell = particles[2][i];
        double force = gravitational_force(r, i, npts, G_CONST, HALO_MASS);
        double dvdt = force + effective_angular_force(r, ell);
        particles[1][i] = vrad + 0.5 * dvdt * dt;
    }
}

int ref_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
