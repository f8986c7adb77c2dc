/*
 * nsg.h -- C ABI of libnsg, the GB300 (sm_103a) implementation of NSphere's
 * per-step shell loop: radial sort -> enclosed mass M(r) and force -> adaptive
 * leapfrog with adaptive Levi-Civita regularisation.
 *
 * The reference (kris-sigurdson/NSphere v0.1.2, src/c/nsphere.c) has no plugin
 * interface: its step is inline code in main().  Each entry point below names
 * the reference code it replaces.  Conventions:
 *   - every call returns NSG_OK (0) or a negative NSG_E* code; the library never
 *     calls exit() (the reference exits through CLEAN_EXIT, nsphere.c:289-298);
 *     nsg_last_error() gives the message of the most recent failure;
 *   - a context owns its device memory and CUDA stream; state stays resident on
 *     the GPU between steps; one context per host thread;
 *   - host arrays are plain pointers to contiguous float64 / int32 columns, laid
 *     out like the reference's particles[component][index] rows
 *     (nsphere.c:4656-4682): 0 = r, 1 = v_r, 2 = ell, 3 = id (stored as double),
 *     4 = mu (carried through the sort when the context was created with
 *     carry_aux = 1);
 *   - there is no CPU fallback: without a usable sm_103a GPU nsg_create fails.
 */
#ifndef NSG_H
#define NSG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSG_OK 0
#define NSG_EINVAL (-1)     /* bad argument (null pointer, n out of range, ...) */
#define NSG_ECUDA (-2)      /* a CUDA runtime call failed */
#define NSG_ENOMEM (-3)     /* device or pinned-host allocation failed */
#define NSG_ESTATE (-4)     /* call out of order (e.g. step before upload) */
#define NSG_EIDS (-5)       /* particle ids are not a permutation of 0..n-1 */
#define NSG_EDEVICE (-6)    /* a kernel reported an error word (see nsg_status) */
#define NSG_ETIMEOUT (-7)   /* nsg_sync timed out */

/* Integration method: the reference's internal method_select codes. */
#define NSG_METHOD_KDK 2          /* fixed-step leapfrog, vel half-step (CLI --method 6), nsphere.c:5484-5559 */
#define NSG_METHOD_ADAPTIVE 3     /* adaptive leapfrog only (CLI --method 3) */
#define NSG_METHOD_FULL_LC 4      /* adaptive leapfrog + fixed-dtau Levi-Civita leapfrog (CLI --method 2),
                                     nsphere.c:5661-5745 with doLeviCivitaLeapfrog :1827-1937; its r_crit
                                     rule has no special case for rank 0 (M_i = 0 there), and the reference
                                     runs it with tol 1e-8, max_subdiv 4096^2 and N_taumin 1000, which the
                                     caller sets in the params */
#define NSG_METHOD_ADAPTIVE_LC 5  /* adaptive leapfrog + adaptive Levi-Civita (CLI --method 1, default), nsphere.c:5775-5838 */

/* Levi-Civita routing rule for NSG_METHOD_ADAPTIVE_LC and NSG_METHOD_FULL_LC. */
#define NSG_LC_RCRIT 0   /* r < alpha * ell^2 / (G M_i), reference rule nsphere.c:5804-5822 */
#define NSG_LC_RADIUS 1  /* r < lc_radius */
#define NSG_LC_OFF 2     /* never */

/* Level scheduling for the adaptive leapfrog. */
#define NSG_SCHED_PLAIN 0    /* try N = 1, 2, 4, ... as the reference does */
#define NSG_SCHED_LEARNED 1  /* start each particle at the level its MLP predicts */

/* Device status bits returned by nsg_status (sticky until nsg_clear_status). */
#define NSG_ST_NAN 0x1u           /* a non-finite radius reached the sort (sorted last) */
#define NSG_ST_TAU_CAP 0x2u       /* a Levi-Civita step hit max_tau_steps */
#define NSG_ST_NOT_CONVERGED 0x4u /* a particle used its last level without converging */
#define NSG_ST_SORT_FALLBACK 0x8u /* the near-sorted bucket sort overflowed; the full radix sort ran */
#define NSG_ST_QUEUE 0x10u        /* a work queue overflowed (internal error) */
#define NSG_ST_IC_REJECT 0x20u    /* an initial-condition rejection loop gave up (nsg_generate) */
#define NSG_ST_DEVICE_WAIT 0x40u  /* a bounded device wait (tensor-core completion) gave up (internal error) */

/* Initial-condition models of nsg_generate. */
#define NSG_IC_PLUMMER 1    /* Plummer sphere, Aarseth-Henon-Wielen speeds */
#define NSG_IC_HERNQUIST 2  /* Hernquist sphere truncated at r_max, isotropic f(E) */

typedef struct nsg_params {
    double G;              /* effective gravitational constant: VEL_CONV_SQ*G_CONST (nsphere.c:365,373); 1 in G=M=1 units */
    double M_total;        /* halo mass: HALO_MASS (nsphere.c:371) */
    double dt;             /* step length */
    double tol_r;          /* relative radius tolerance, 1e-7 (nsphere.c:5778) */
    double tol_v;          /* relative velocity tolerance, 1e-7 (nsphere.c:5777) */
    int64_t max_subdiv;    /* largest subdivision N tried; reference 4096*4096*16 (nsphere.c:5779) */
    int32_t out_type;      /* 0 coarse, 1 fine, 2 Richardson 4F-3C (nsphere.c:5780) */
    int32_t N_taumin;      /* tau-steps target of the Levi-Civita guess, 10 (nsphere.c:5781) */
    int32_t method;        /* NSG_METHOD_* */
    int32_t lc_rule;       /* NSG_LC_* */
    double lc_alpha;       /* 0.05 (nsphere.c:5782) */
    double lc_radius;      /* radius for NSG_LC_RADIUS */
    int64_t max_tau_steps; /* Levi-Civita tau-step cap, 1e8 (nsphere.c:2273) */
    int32_t sched;         /* NSG_SCHED_* */
    int32_t carry_aux;     /* 1: permute a fifth float64 column (mu) with the state */
    int32_t sort_mode;     /* 0 auto (near-sorted bucket sort, radix fallback), 1 always radix */
    int32_t graph;         /* 1: repeat steps by replaying a captured CUDA graph of two steps (default) */
    double point_mass;     /* central point mass added to M_i at the step start (0 = reference) */
    double point_mass_rate;/* d(point_mass)/dt, applied per step (linear ramp) */
    int32_t nonfinite_stop;/* 1 (default): a pass with a non-finite radius or velocity ends the
                              level climb, and a non-finite Levi-Civita state ends the particle's
                              tau-steps; 0: follow the reference, which keeps climbing (up to
                              max_subdiv) and stepping (up to max_tau_steps) on such values */
    int32_t reserved;
} nsg_params;

typedef struct nsg_ctx nsg_ctx;

/* Per-kernel timing accumulated while profiling is on (CUDA events on the
 * context's stream). */
typedef struct nsg_kernel_stat {
    char name[32];
    int64_t launches;
    double total_ms;
    double bytes;          /* algorithmic bytes moved by those launches */
} nsg_kernel_stat;

/* Fills the reference's method-5 defaults in G=M=1 units (dt 5e-4, tol 1e-7,
 * max_subdiv 2^28, out_type 2, N_taumin 10, r_crit rule with alpha 0.05). */
int nsg_params_default(nsg_params *p);

/* Creates a context on the current CUDA device.  stream may be NULL (the
 * context creates its own) or a cudaStream_t the caller owns. */
int nsg_create(nsg_ctx **ctx, const nsg_params *p, void *stream);
void nsg_destroy(nsg_ctx *ctx);
const char *nsg_last_error(nsg_ctx *ctx);   /* ctx may be NULL: last global error */
int nsg_set_params(nsg_ctx *ctx, const nsg_params *p);
int nsg_get_params(nsg_ctx *ctx, nsg_params *p);

/* Uploads the state from host columns (the reference's particles[0..3][0..n-1];
 * aux = particles[4], may be NULL).  ids must be a permutation of 0..n-1, as the
 * reference's inverse_map requires (nsphere.c:5789-5794).  Replaces nothing in the
 * reference (its state is host-resident); the upload is the one H2D copy. */
int nsg_upload(nsg_ctx *ctx, const double *r, const double *vr, const double *ell,
               const double *id_as_double, const double *aux, int64_t n);
/* Ensemble of independent halos (no reference counterpart: the reference runs one
 * halo per process).  Halo h is the next halo_n[h] rows of the columns; every halo
 * is sorted, ranked (M_i = (i/N_h) M with its own N_h) and integrated on its own in
 * the same launches.  ids: a permutation of 0..n-1 in which halo h owns the ids of
 * its own row range. */
int nsg_upload_ensemble(nsg_ctx *ctx, const double *r, const double *vr, const double *ell,
                        const double *id_as_double, const double *aux, const int64_t *halo_n,
                        int nhalo);
int nsg_num_halos(nsg_ctx *ctx);
/* Per-halo energies K[h], W[h] (arrays of nsg_num_halos entries). */
int nsg_energy_halos(nsg_ctx *ctx, double *K, double *W);
/* Same with the reference's double ** row table: particles[0..4]. */
int nsg_upload_particles(nsg_ctx *ctx, double *const *particles, int64_t n);
/* Same from device pointers (int32 ids). */
int nsg_upload_device(nsg_ctx *ctx, const double *d_r, const double *d_vr,
                      const double *d_ell, const int32_t *d_id, const double *d_aux,
                      int64_t n);

/* Runs nsteps full steps of params.method.  Replaces the body of the time loop at
 * nsphere.c:5775-5838 (method 5) / :5484-5531 (method 2): sort_particles
 * (nsphere.c:8662), the inverse_map rebuild, and the per-particle integrators
 * doAdaptiveFullLeap (nsphere.c:1648) / doAdaptiveFullLeviCivita (nsphere.c:2231). */
int nsg_step(nsg_ctx *ctx, int nsteps);

/* Sorts the resident state by (r, id) -- sort_particles (nsphere.c:8662) -- and
 * computes the rank force numerators.  Idempotent. */
int nsg_sort(nsg_ctx *ctx);

/* Downloads the state in its current array order (after nsg_step: the order of
 * the sort at the start of the last step, as the reference's particles array). */
int nsg_download(nsg_ctx *ctx, double *r, double *vr, double *ell,
                 double *id_as_double, double *aux);
int nsg_download_particles(nsg_ctx *ctx, double *const *particles);
/* nsteps steps followed by nsg_download, with the same results: in the last step the
 * copy of the particles the leapfrog kernels integrate runs beside the Levi-Civita
 * chains, and the chains' particles are patched in when they end (no reference
 * counterpart; a driver that downloads every step, like the snapshot code at
 * nsphere.c:6452, hides most of the copy this way). */
int nsg_step_download(nsg_ctx *ctx, int nsteps, double *r, double *vr, double *ell,
                      double *id_as_double, double *aux);
/* Device-pointer views of the resident columns (valid until the next call). */
int nsg_device_state(nsg_ctx *ctx, double **d_r, double **d_vr, double **d_ell,
                     int32_t **d_id, int64_t *n);

/* Stateless drop-in for sort_particles(double **particles, int npts)
 * (nsphere.c:8662): uploads the five columns, sorts on the GPU by (r, id),
 * downloads them permuted.  Uses ctx's buffers and stream. */
int nsg_sort_particles(nsg_ctx *ctx, double *const *particles, int64_t npts);

/* Allocation-free variant of the sort (no counterpart in the reference, whose sort
 * runs on host arrays): sorts caller-owned DEVICE columns in place by (r, id) --
 * ties by id, then input position -- with no context and no device allocation,
 * its scratch being one fixed 34,078,720-byte __device__ array per device.
 * npts > 1048576 returns NSG_EINVAL untouched; aux may be NULL; work is queued
 * on `stream` (a cudaStream_t of the current device, NULL = legacy default).  A call
 * outside stream capture looks the scratch address up (cudaGetSymbolAddress), so it
 * follows a device reset or a new context; a call made while `stream` is being
 * captured reuses the address of the last call on the device, so the first call on a
 * device should come before any capture.  A CUDA error pending from earlier work is
 * returned (NSG_ECUDA) without running the sort.  Calls that overlap in time on one
 * device share the scratch and race: keep them on one stream. */
int nsg_sort_device_noalloc(double *d_r, double *d_vr, double *d_ell, int32_t *d_id, double *d_aux,
                            int64_t npts, void *stream);

/* Generates n particles of a seeded model on the GPU into the resident state (G = M =
 * a = 1, ids = radial rank, mu in the fifth column when carry_aux), in place of the
 * reference's GSL-based generators (nsphere.c:4238-4824); r_max is the Hernquist
 * truncation radius (ignored for Plummer).  Counter-based draws: the result depends
 * only on (model, n, seed, r_max). */
int nsg_generate(nsg_ctx *ctx, int model, int64_t n, uint64_t seed, double r_max);
/* The Hernquist model with Osipkov-Merritt anisotropy of radius r_a (the reference
 * builds its models from GSL splines of the distribution function,
 * nsphere.c:4238-4824): f(Q) = f_iso(Q) + sqrt(Q) (1 - 2Q) / (sqrt(2) pi^3 r_a^2), the
 * closed-form Eddington inversion of rho_Q = (1 + r^2/r_a^2) rho. */
int nsg_generate_om(nsg_ctx *ctx, int64_t n, uint64_t seed, double r_max, double r_a);

/* Per-particle potential and energy of the post-processing (nsphere.c:7697-7846), on
 * the resident state in its sorted order (sorted first if needed; one halo):
 * psi[i] = G (M_i / r_i + dM sum_{j>i} 1/r_j) with M_i = (i+1) dM, dM = M_total / N;
 * E[i] = psi[i] - ell_i^2/(2 r_i^2) - v_i^2/2; *psi0 = G dM sum_j 1/r_j.  psi, E are
 * host arrays of n doubles (either may be NULL); the suffix sums are a parallel scan,
 * so values agree with the reference's sequential sums to rounding. */
int nsg_potential(nsg_ctx *ctx, double *psi, double *E, double *psi0);

/* Records of the reference's Rank files, written with fprintf_bin (nsphere.c:2550-2588:
 * %d as int32, %f as float), Rank_Mass_Rad_VRad_sorted_t*.dat (nsphere.c:7966-7983)
 * and Rank_Mass_Rad_VRad_unsorted_t*.dat (:7930-7945). */
typedef struct nsg_rank_sorted {
    int32_t rank; float mass, r, vr, psi, E, ell, rho;
} nsg_rank_sorted;
typedef struct nsg_rank_unsorted {
    int32_t rank; float mass, r, vr, psi, E, ell;
} nsg_rank_unsorted;

/* Per-snapshot post-processing of nsphere.c:7060-7990 on the GPU.  records holds the n
 * 16-byte snapshot records {int32 rank, float r, v_r, ell} of one all_particle_data
 * block (nsphere.c:1295-1324, record order = particle order).  The records become the
 * context's resident state (NaN r and v_r read as 0, :7112-7119; ids = record index)
 * and are sorted by (r, record index); the reference's qsort leaves the order of equal
 * radii unspecified.  Outputs (host, either may be NULL): sorted_out[n] -- sorted
 * position, M = (i+1) M_total/n, r, v_r, Psi_A, E, ell and the smoothed density of
 * :7281-7686 -- and unsorted_out[n] in record order; *psi0 = Psi_A(0).
 *   Psi_A at the sorted radii are the knots of a linear interpolation evaluated at
 *   every radius, with the knots 0, r_0, ..., r_{n-1} made strictly increasing by
 *   moving each knot not above its predecessor to the predecessor + 1e-5 (:7752-7768).
 *   The density: M(r) of the strictly increasing radii, decimated to
 *   min(ceil(n/100), 30000) points, natural cubic spline onto 131072 log-spaced radii,
 *   dM/dr by central differences (floor 1e-10), smoothed in log r by the normalised
 *   one-sided Gaussian of width 0.08 (n/1e4)^-0.4 that the reference's zero-padded FFT
 *   convolution applies (:2901-3104; summed directly here), and splined back to the
 *   particles.  NSG_EINVAL when the density is undefined (fewer than 3 distinct
 *   radii after decimation, or a smallest radius <= 0). */
int nsg_post_snapshot(nsg_ctx *ctx, const void *records, int64_t n, nsg_rank_sorted *sorted_out,
                      nsg_rank_unsorted *unsorted_out, double *psi0);

/* The initial-conditions file of write_initial_conditions / read_initial_conditions
 * (nsphere.c:2386-2487): int32 npts, then npts records of five doubles (r, v_r, ell,
 * original index, mu).  nsg_write_init writes the resident state in its current
 * order (mu = 0 unless carry_aux); nsg_read_init uploads a file's state like
 * nsg_upload (expected_n < 0 accepts any count; otherwise a different count is an
 * error, where the reference prints a warning and keeps its arrays). */
int nsg_write_init(nsg_ctx *ctx, const char *filename);
int nsg_read_init(nsg_ctx *ctx, const char *filename, int64_t expected_n);

/* The all_particle_data stream (nsphere.c:1295-1324, 6452-6564).  Each nsg_snapshot
 * appends, for every particle in original-id order, a 16-byte record {int32 rank
 * in the last sort, float r, float v_r, float ell} of the resident state; records are
 * packed on the GPU and written by a background thread while later steps run (two
 * snapshots in flight; a third waits).  nsg_snapshot_close drains and closes. */
int nsg_snapshot_open(nsg_ctx *ctx, const char *filename, int append);
int nsg_snapshot(nsg_ctx *ctx);
int nsg_snapshot_close(nsg_ctx *ctx);

/* Looks up k particles by id -- the inverse_map reads of the tracking code
 * (nsphere.c:5845-5866, 6384-6450).  rank receives the current array index. */
int nsg_gather(nsg_ctx *ctx, const int32_t *ids, int k, double *r, double *vr,
               double *ell, int32_t *rank);

/* Static potential of the initial halo for the tracking energies.  The reference
 * tabulates Psi(r) = G M(r)/r + G int_r^inf 4 pi r' rho dr' of its mass-normalised
 * profile on a 10000-point grid and evaluates a cubic spline of it
 * (nsphere.c:4575-4592, evaluatespline :8205-8236); here Psi is the closed form of the
 * same integrals.  NSG_PSI_CORED is the reference's own profile
 * rho ~ (1 + r^2/a^2)^-3 (massintegrand, nsphere.c:8157-8161; a = RC, r_trunc = 10 RC). */
#define NSG_PSI_CORED 0
#define NSG_PSI_PLUMMER 1      /* rho ~ (1 + r^2/a^2)^-5/2 */
#define NSG_PSI_HERNQUIST 2    /* rho ~ 1 / (r/a (1 + r/a)^3) */

typedef struct nsg_psi {
    int32_t model;      /* NSG_PSI_* */
    int32_t reserved;
    double a;           /* scale radius (RC for the cored profile) */
    double r_trunc;     /* radius the mass is normalised within (rmax, nsphere.c:4528); <= 0: untruncated */
    double r_lo, r_hi;  /* table range: r < r_lo is evaluated at r_lo + 1e-10, r > r_hi at r_hi - 1e-10
                           (the reference's grid is [0, 0.9999 rmax]); r_hi <= 0: no upper clamp */
} nsg_psi;

/* Device-side trajectory recorder: the per-step tracking of nsphere.c:6384-6450
 * without a host round trip.  After every step (inside the captured step graph) the
 * k particles ids[0..k) are looked up through the inverse map and
 *   r, v_r, ell, E_rel = Psi(r) - (v_r^2 + ell^2/r^2)/2, mu = v_r / sqrt(v_r^2 + ell^2/r^2)
 * are stored for the next of `capacity` step slots.  The last k_clamped ids are the
 * low-ell group of :6414-6444, whose radius is first clamped (r < 0 -> 1e-10,
 * r > r_trunc -> r_trunc) and stored clamped.  G and M are the context's.  Steps after
 * the buffer is full are counted but not stored.  An id outside [0, n) records NaN.
 * Opening again replaces the recorder. */
int nsg_track_open(nsg_ctx *ctx, const int32_t *ids, int k, int k_clamped, const nsg_psi *psi,
                   int64_t capacity);
/* Copies the records into out[5][k][capacity] (r, v_r, ell, E_rel, mu; step slot
 * fastest).  recorded = slots filled, steps_seen = steps since the open. */
int nsg_track_read(nsg_ctx *ctx, double *out, int64_t *recorded, int64_t *steps_seen);
int nsg_track_close(nsg_ctx *ctx);

/* Total energy of the resident state, K = sum 1/2 m (v_r^2 + ell^2/r^2) and
 * W = sum m G_num(i)/r_i with the rank enclosed mass of nsphere.c:513.  Sorts the
 * state first (the sort is a total order, so later steps are unaffected). */
int nsg_energy(nsg_ctx *ctx, double *K, double *W);

/* Histogram of accepted adaptive-leapfrog levels of the last step: hist[k] for
 * k < nbins-2; hist[nbins-2] = particles that never converged; hist[nbins-1] =
 * particles integrated by Levi-Civita. */
int nsg_level_hist(nsg_ctx *ctx, int64_t *hist, int nbins);
/* Per-particle accepted level of the last step (int8, -1 = not converged,
 * 100+k / 99 = Levi-Civita), in current array order. */
int nsg_levels(nsg_ctx *ctx, int8_t *levels);

int nsg_sync(nsg_ctx *ctx, int timeout_ms);
int nsg_status(nsg_ctx *ctx, uint32_t *flags);
int nsg_clear_status(nsg_ctx *ctx);

/* Diagnostic without a reference counterpart: compares the library's integer-pipe
 * double divisions (used by every integrator in place of the FP64 pipe's) with the
 * hardware IEEE division on `count` generated operand pairs on the current device,
 * and its division-free test RN(|a|/|b|) < tol (the integrators' acceptance tests)
 * with the divided quotient, for tol at, one ulp either side of, and away from the
 * quotient.  mismatches must come back 0; fast_path counts pairs that took the
 * integer path; first_bad[0..1] receives the first mismatching (a, b). */
int nsg_selftest_division(uint64_t seed, int64_t count, int64_t *mismatches,
                          int64_t *fast_path, double *first_bad);

/* Diagnostic without a reference counterpart: FP64 figures of the current device
 * used as roofline denominators for the FP64-bound integrators (any pointer may be
 * NULL): FMA throughput in TFLOP/s, IEEE division throughput on the FP64 pipe and on
 * the integer pipe in G divisions/s, and single-warp dependent latency of one FMA
 * and one division in cycles. */
int nsg_probe_fp64(double *dfma_tflops, double *div_hw_gps, double *div_int_gps,
                   double *fma_latency_cycles, double *div_latency_cycles);
/* Dependent latencies in cycles per iteration, one block on one SM (no reference
 * counterpart): cycles[0] FP64 FMA chain; [1] two independent FMA chains in one warp;
 * [2] one chain in each of two warps; [3] dadd + FP64-pipe division; [4] dadd +
 * the throughput kernels' division (latency form, fallback behind a call); [5] dadd +
 * latency-oriented division;
 * [6] 32-bit integer multiply-add; [7] 64-bit multiply-high; [8] int->float, multiply,
 * float->int; [9] one Levi-Civita substep of the leading warp (split force); [10] the
 * same with a zero gravity numerator; [11] the same with both force quotients in
 * every lane (no exchange); [12] dadd of a value and its copy from the other half of
 * the warp (shuffle); [13] dadd, then a 64-bit select by lane half.  count = how many
 * to measure (<= 14). */
int nsg_probe_latency(double *cycles, int count);

/* ---- learned level scheduler (no reference counterpart: an addition of this
 * library).  A 4 -> 64 -> 64 -> 8 MLP with BF16 weights and FP32 accumulation
 * predicts from (r, v_r, ell, local dynamical time) the adaptive-leapfrog level each
 * particle will accept.  With params.sched = NSG_SCHED_LEARNED a particle predicted
 * to need level >= 1 skips the level-0 pass; every level is still tested from 0
 * upward, so results are bit-identical to NSG_SCHED_PLAIN.  Predictions are made on
 * the tensor cores from the state as a step starts; a learned step of one halo under
 * NSG_LC_RADIUS makes the next step's at its own end, beside its Levi-Civita chains.
 * Changing the weights (init, set, train) or the state (upload, sort) makes the next
 * step predict afresh. */
int nsg_mlp_num_params(void);
/* Random initial weights (seeded); allocates the network on the context. */
int nsg_mlp_init(nsg_ctx *ctx, uint64_t seed);
int nsg_mlp_set_weights(nsg_ctx *ctx, const float *w, int64_t count);
int nsg_mlp_get_weights(nsg_ctx *ctx, float *w, int64_t count);
/* Runs nsteps plain adaptive steps and appends (features, accepted level) of every
 * particle that needed level >= 1 and of level-0 particles with probability
 * keep_level0 to a device-resident training set of `capacity` samples. */
int nsg_mlp_collect(nsg_ctx *ctx, int nsteps, double keep_level0, int64_t capacity);
/* Size of the training set (and up to max samples copied to X[.][4], y[.]). */
int nsg_mlp_dataset(nsg_ctx *ctx, int64_t *count, float *X, int8_t *y, int64_t max);
/* Adam on the GPU over the training set (level-0 samples weighted 1/keep_level0). */
int nsg_mlp_train(nsg_ctx *ctx, int epochs, int batch, float lr, uint64_t seed, double *final_loss);
/* Forward + backward of the class-weighted softmax cross-entropy summed over nb
 * samples; grad receives nsg_mlp_num_params() floats (summed over samples). */
int nsg_mlp_grad(nsg_ctx *ctx, const float *X, const int8_t *y, int64_t nb, const float *cls_w,
                 float *grad, double *loss);
/* Predicted class (and the 8 logits, may be NULL) of nb feature vectors. */
int nsg_mlp_predict(nsg_ctx *ctx, const float *X, int64_t nb, int8_t *cls, float *logits);

/* Kernels launched by steps and sorts so far, and steps taken (for reporting). */
int nsg_counters(nsg_ctx *ctx, int64_t *launches, int64_t *steps);

int nsg_profile(nsg_ctx *ctx, int enable);
int nsg_profile_read(nsg_ctx *ctx, nsg_kernel_stat *stats, int max, int *count);

/* Launch-shape tuning (no counterpart in the reference, whose step runs on CPU
 * threads).  vals[4] = {gather_level0 threads (128|256|512), gather_level0 blocks
 * per SM (1..64), log2 of sorted positions per bucket (8..12; 9..11 sort inside the
 * kernel that consumes the sort, 8 and 12 with a separate bucket-sort kernel),
 * level-kernel blocks per SM (1..64)}.  Shapes change no arithmetic: results are
 * identical for every setting. */
int nsg_tune_get(nsg_ctx *ctx, int32_t *vals, int count);
int nsg_tune_set(nsg_ctx *ctx, const int32_t *vals, int count);
/* Times candidate shapes over `steps` steps of the resident state, one knob at a
 * time, keeps the fastest and restores the state, step count and status exactly.
 * A JSON summary of the timings is written to report (may be NULL). */
int nsg_autotune(nsg_ctx *ctx, int steps, char *report, int report_cap);

#ifdef __cplusplus
}
#endif
#endif /* NSG_H */
