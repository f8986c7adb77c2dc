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
#endif
