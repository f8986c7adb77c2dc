/* nsg_oracle.h -- CPU oracle of the NSphere step loop (test infrastructure only). */
#ifndef NSG_ORACLE_H
#define NSG_ORACLE_H
#include <stdint.h>

typedef struct orc_params {
    double G;              /* effective G: the reference's VEL_CONV_SQ * G_CONST */
    double M;              /* halo mass, the reference's HALO_MASS */
    double dt;             /* step */
    double tol_r, tol_v;   /* relative coarse/fine tolerances (reference 1e-7) */
    int64_t max_subdiv;    /* largest N tried (reference 2^28) */
    int out_type;          /* 0 coarse, 1 fine, 2 Richardson 4F-3C */
    int N_taumin;          /* Levi-Civita tau-steps target (reference 10) */
    int lc_rule;           /* 0: r < alpha*ell^2/(G M_i); 1: r < lc_radius; 2: never */
    double lc_alpha;       /* 0.05 */
    double lc_radius;      /* 1e-3 */
    int64_t max_tau_steps; /* tau-step cap (reference 1e8) */
    double point_mass;     /* central point mass added to M_i (not in the reference; 0 = reference) */
    int nonfinite_stop;    /* 1: a non-finite pass ends the climb / the tau-steps; 0: the reference */
    int lc_fixed;          /* 1: method 4 (fixed-dtau Levi-Civita leapfrog, r_crit without the rank-0 case) */
} orc_params;

void orc_params_default(orc_params *p);
double orc_gnum(int64_t i, int64_t n, double G, double M);
double orc_gnum_pm(int64_t i, int64_t n, double G, double M, double Mpt);
void orc_micro_leap(double r_in, double v_in, double l2, double gnum, double h,
                    int64_t N, int fine, double *r_out, double *v_out);
void orc_adaptive_leap(double r_in, double v_in, double ell, double gnum, double h,
                       double tol_r, double tol_v, int64_t max_subdiv, int out_type,
                       double *r_out, double *v_out, int *level);
int orc_adaptive_lc(double r_in, double v_in, double ell, double gnum, double dt,
                    int N_taumin, double tol_r, double tol_v, int64_t max_subdiv,
                    int out_type, int64_t max_tau_steps,
                    double *r_out, double *v_out, int *level, int64_t *ntau);
int orc_sort(int64_t n, double *r, double *vr, double *ell, int32_t *id, double *aux);
int64_t orc_step_adaptive(const orc_params *p, int64_t n, double *r, double *vr,
                          double *ell, int32_t *id, int8_t *level);
void orc_step_kdk(const orc_params *p, int64_t n, double *r, double *vr, double *ell,
                  int32_t *id);
void orc_energy(const orc_params *p, int64_t n, const double *r, const double *vr,
                const double *ell, double *K, double *W);
int orc_num_threads(void);
/* Fixed-dtau Levi-Civita leapfrog over physical dt, nsphere.c:1827-1937 (returns 1 when
 * the step cap was hit). */
int orc_lc_fixed(double r_in, double v_in, double ell, double gnum, double dt, int N_taumin,
                 int64_t max_steps, double *r_out, double *v_out);
/* Static halo potential of the tracking energies (nsphere.c:4575-4592, 8205-8236):
 * model 0 cored (1+x^2)^-3, 1 Plummer, 2 Hernquist; r_trunc <= 0 untruncated;
 * r < r_lo is evaluated at r_lo + 1e-10 and r > r_hi (> 0) at r_hi - 1e-10. */
double orc_psi(int model, double a, double r_trunc, double r_lo, double r_hi, double G, double M, double r);
/* One step's tracking records (nsphere.c:6384-6450) of k particles given their
 * r, v_r, ell: out[5][k] = r (clamped for the last k_clamped), v_r, ell, E_rel, mu. */
void orc_track(int model, double a, double r_trunc, double r_lo, double r_hi, double G, double M,
               int k, int k_clamped, const double *r, const double *vr, const double *ell, double *out);
/* Per-snapshot post-processing (nsphere.c:7060-7990).
 * orc_density: smoothed density at each of n sorted radii whose enclosed masses are
 * (i+1) M/n (returns 0, or -1 when the radii are rejected).
 * orc_psi_knots: the n+1 knots of the Psi_A interpolation.
 * orc_post_snapshot: the rank-file quantities of float records r, v, ell in record
 * order -- sorted by (r, record index): s_idx, s_r, s_v, s_l, s_psi, s_E, s_rho;
 * record order: u_psi, u_E -- with Psi_A(0) in psi0 (returns orc_density's status). */
int orc_density(int64_t n, const double *R, double M, double *rho);
void orc_psi_knots(int64_t n, const double *R, double *knots);
int orc_post_snapshot(int64_t n, const float *r, const float *v, const float *l, double G, double M,
                      int64_t *s_idx, double *s_r, double *s_v, double *s_l, double *s_psi, double *s_E,
                      double *s_rho, double *u_psi, double *u_E, double *psi0);
#endif
