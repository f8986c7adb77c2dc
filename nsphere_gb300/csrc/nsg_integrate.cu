// nsg_integrate.cu -- per-particle integrators of the step, on the sorted state.
//
// Adaptive leapfrog (nsphere.c:1550-1735) as per-level work queues:
//   level 0 runs for every particle (coarse N=1 and fine N=1);
//   level k >= 1 runs only for the particles queued by level k-1.
// Two facts keep the results bit-identical to the reference's loop:
//   * every level restarts from the step's initial (r, v) (nsphere.c:1673-1684),
//     so a particle at level k needs only its inputs;
//   * the coarse pass of level k (2N'+1 substeps, N' = 2^k) performs exactly the
//     operations of the fine pass of level k-1 (4N+1 substeps, N = 2^(k-1)):
//     halfKick h/(2N') = h/(4N) and midStep h/N' = h/(2N).  The queue therefore
//     carries the previous fine result and level k computes only its fine pass.
// The first force of every pass is the force at (r_in, rank) that the rank/force
// pass already wrote (a0), as every pass starts with the same half-kick at r_in.
//
// Levi-Civita particles (nsphere.c:1990-2334) are listed by level 0 and integrated
// on a side stream, overlapped with the leapfrog levels.
#include "nsg_internal.cuh"

namespace nsg {

struct StepArgs {
    // sorted copy: the fused gather writes start values here; every particle's
    // final (r, v) overwrites them in place once its level is accepted
    const double *r_in, *v_in, *ell;
    double *a0;                 // written for queued particles only
    double *r_out, *v_out;      // alias r_in / v_in
    double *ell_out, *aux_out;
    int32_t *id_out, *inv;
    // unsorted source copy and the permutation from the radix sort
    const uint32_t *perm;
    const double *r_src, *v_src, *l_src, *aux_src;
    const int32_t *id_src;
    int8_t *level;
    int64_t n;
    double G, M, dt, tol_r, tol_v;
    int64_t max_subdiv;
    int nlev;                   // number of levels: floor(log2(max_subdiv)) + 1
    int out_type;
    int method;
    int lc_rule;
    double lc_alpha, lc_radius;
    int N_taumin;
    int64_t max_tau_steps;
    DevCounters *ctr;
    uint32_t *q_idx[2];
    double *q_r[2], *q_v[2];
    uint32_t *lc_idx;
    // Substep sizes of each pass, identical for every particle, computed once on
    // the host with the same IEEE divisions as nsphere.c:1566-1577:
    // coarse N=1: halfKick h/(2.0*1), midStep h/(1.0*1); fine N=2^k: h/(4.0*N), h/(2.0*N).
    double hk_c0, ms_c0;
    double hk_f[kMaxLevels], ms_f[kMaxLevels];
};

// Micro leapfrog, nsphere.c:1550-1607: half-kick, (pairs-1) drift-kick pairs, drift,
// half-kick.  pairs = N (coarse, 2N+1 substeps) or 2N (fine, 4N+1 substeps); the
// first acceleration a_first = acc(r_in) is supplied by the rank/force pass.
__device__ __forceinline__ void micro_leap(double r, double v, double l2, double gn,
                                           double hk, double ms, int64_t pairs, double a_first,
                                           double &r_out, double &v_out)
{
    v = dadd(v, dmul(hk, a_first));
    for (int64_t pp = 1; pp <= pairs - 1; pp++) {
        r = dadd(r, dmul(ms, v));
        v = dadd(v, dmul(ms, acc_leap(r, gn, l2)));
    }
    r = dadd(r, dmul(ms, v));
    v = dadd(v, dmul(hk, acc_leap(r, gn, l2)));
    r_out = r;
    v_out = v;
}

__device__ __forceinline__ bool converged(double rc, double vc, double rf, double vf,
                                          double tol_r, double tol_v)
{
    double dr = ddiv(fabs(dsub(rf, rc)), dadd(fabs(rf), 1.0e-30));
    double dv = ddiv(fabs(dsub(vf, vc)), dadd(fabs(vf), 1.0e-30));
    return (dr < tol_r) && (dv < tol_v);
}

__device__ __forceinline__ void select_out(int out_type, double rc, double vc, double rf,
                                           double vf, double &ro, double &vo)
{
    if (out_type == 0) { ro = rc; vo = vc; }
    else if (out_type == 1) { ro = rf; vo = vf; }
    else {
        ro = dsub(dmul(4.0, rf), dmul(3.0, rc));
        vo = dsub(dmul(4.0, vf), dmul(3.0, vc));
    }
}

// Routing of nsphere.c:5804-5822 (alpha rule), or a fixed radius.
__device__ __forceinline__ bool route_lc(const StepArgs &a, int64_t i, double r, double ell)
{
    if (a.method != NSG_METHOD_ADAPTIVE_LC || a.lc_rule == NSG_LC_OFF) return false;
    if (a.lc_rule == NSG_LC_RADIUS) return (r > 1.0e-30) && (r < a.lc_radius);
    double r_crit = 0.0;
    if (fabs(ell) > 1.0e-30) {
        double M_enc;
        if (i == 0) M_enc = dmul(dmul(0.1, ddiv(1.0, (double)a.n)), a.M);
        else M_enc = dmul(ddiv((double)i, (double)a.n), a.M);
        double gravPart = dmul(a.G, M_enc);
        r_crit = ddiv(dmul(dmul(ell, ell), a.lc_alpha), gravPart);
    }
    return (r > 1.0e-30) && (r < r_crit);
}

// Fused pass after the radix sort, per sorted position i: gather the particle
// into sorted order, write the inverse map (nsphere.c:5789-5794), compute its
// rank force numerator and start acceleration (nsphere.c:502-535), route it
// (nsphere.c:5804-5822), and run adaptive level 0 (nsphere.c:1660-1700).  The
// pass is FP64-bound, so the gather traffic hides under the arithmetic.
template <bool AUX>
__global__ void __launch_bounds__(256) k_gather_level0(StepArgs a)
{
    const double Mpt = a.ctr->point_mass;
    const bool last = (a.nlev <= 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = a.perm[i];
        double r = a.r_src[s], v = a.v_src[s], ell = a.l_src[s];
        const int32_t idv = a.id_src[s];
        a.ell_out[i] = ell;
        a.id_out[i] = idv;
        if (AUX) a.aux_out[i] = a.aux_src[s];
        a.inv[idv] = (int32_t)i;
        bool lc = route_lc(a, i, r, ell);
        int slot = warp_append(lc, &a.ctr->lc_count);
        if (lc) {
            a.r_out[i] = r;          // start values for the Levi-Civita kernel
            a.v_out[i] = v;
            a.lc_idx[slot] = (uint32_t)i;
            continue;
        }
        double gn = gnum_of(i, a.n, a.G, a.M, Mpt);
        double l2 = dmul(ell, ell);
        double af = acc_leap(r, gn, l2);
        double rc, vc, rf, vf;
        micro_leap(r, v, l2, gn, a.hk_c0, a.ms_c0, 1, af, rc, vc);
        micro_leap(r, v, l2, gn, a.hk_f[0], a.ms_f[0], 2, af, rf, vf);
        bool ok = converged(rc, vc, rf, vf, a.tol_r, a.tol_v);
        bool bad = !(isfinite(rf) && isfinite(vf));
        bool done = ok || last || bad;
        if (done) {
            double ro, vo;
            select_out(a.out_type, rc, vc, rf, vf, ro, vo);
            a.r_out[i] = ro;
            a.v_out[i] = vo;
            a.level[i] = ok ? 0 : kLevelNotConverged;
            if (!ok) atomicOr(&a.ctr->status, bad ? (NSG_ST_NAN | NSG_ST_NOT_CONVERGED) : NSG_ST_NOT_CONVERGED);
        }
        int q = warp_append(!done, &a.ctr->qcount[1]);
        if (!done) {
            a.r_out[i] = r;          // start values stay for the higher levels
            a.v_out[i] = v;
            a.a0[i] = af;
            a.q_idx[1][q] = (uint32_t)i;
            a.q_r[1][q] = rf;
            a.q_v[1][q] = vf;
        }
    }
}

// Level k >= 1 over the entries queued by level k-1.
__global__ void __launch_bounds__(256) k_level(StepArgs a, int k)
{
    const unsigned cnt = a.ctr->qcount[k];
    if (cnt == 0) return;
    const double Mpt = a.ctr->point_mass;
    const bool last = (k >= a.nlev - 1);
    const int qi = k & 1, qo = (k + 1) & 1;
    const int64_t pairs = (int64_t)2 << k;   // fine pass of N = 2^k: 2N pairs
    const double hk = a.hk_f[k], ms = a.ms_f[k];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < cnt;
         e += (int64_t)gridDim.x * blockDim.x) {
        uint32_t i = a.q_idx[qi][e];
        double rc = a.q_r[qi][e], vc = a.q_v[qi][e];
        double r = a.r_in[i], v = a.v_in[i], ell = a.ell[i];
        double gn = gnum_of(i, a.n, a.G, a.M, Mpt);
        double l2 = dmul(ell, ell);
        double rf, vf;
        micro_leap(r, v, l2, gn, hk, ms, pairs, a.a0[i], rf, vf);
        bool ok = converged(rc, vc, rf, vf, a.tol_r, a.tol_v);
        bool bad = !(isfinite(rf) && isfinite(vf));
        bool done = ok || last || bad;
        if (done) {
            double ro, vo;
            select_out(a.out_type, rc, vc, rf, vf, ro, vo);
            a.r_out[i] = ro;
            a.v_out[i] = vo;
            a.level[i] = ok ? (int8_t)k : (int8_t)kLevelNotConverged;
            if (!ok) atomicOr(&a.ctr->status, bad ? (NSG_ST_NAN | NSG_ST_NOT_CONVERGED) : NSG_ST_NOT_CONVERGED);
        }
        int q = warp_append(!done, &a.ctr->qcount[k + 1]);
        if (!done) {
            a.q_idx[qo][q] = i;
            a.q_r[qo][q] = rf;
            a.q_v[qo][q] = vf;
        }
    }
}

// ---------------------------------------------------------- Levi-Civita path

// subSteps tau-leapfrog substeps over h_tau, nsphere.c:1990-2036.
__device__ __forceinline__ void micro_lc(double rho, double v, double t, int64_t subSteps,
                                         double h_tau, double gn, double l2,
                                         double &rho_o, double &v_o, double &t_o)
{
    const double dtau = ddiv(h_tau, (double)subSteps);
    const double hdt = dmul(0.5, dtau);
    for (int64_t ss = 0; ss < subSteps; ss++) {
        double f1 = acc_lc(rho, gn, l2);
        double vh = dadd(v, dmul(hdt, f1));
        double rn = dadd(rho, dmul(dtau, dmul(dmul(0.5, rho), vh)));
        double f2 = acc_lc(rn, gn, l2);
        double vn = dadd(vh, dmul(hdt, f2));
        double rm = dmul(0.5, dadd(rho, rn));
        t = dadd(t, dmul(dtau, dmul(rm, rm)));
        rho = rn;
        v = vn;
    }
    rho_o = rho; v_o = v; t_o = t;
}

// One adaptive tau-step, nsphere.c:2077-2186.  The coarse pass of level k is the
// fine pass of level k-1 (same substep count over the same h_tau).  Returns the
// accepted level or -1 (fallback fine pass at 4*(2*N_last)+1 substeps).
__device__ int tau_step_lc(double rho, double v, double t, double hg, double tol_r,
                           double tol_v, int nlev, double gn, double l2, int out_type,
                           double &rho_o, double &v_o, double &t_o)
{
    double rC, vC, tC, rF, vF, tF;
    micro_lc(rho, v, t, 3, hg, gn, l2, rC, vC, tC);
    int64_t N = 1;
    for (int k = 0; k < nlev; k++, N *= 2) {
        micro_lc(rho, v, t, 4 * N + 1, hg, gn, l2, rF, vF, tF);
        double rsq = dmul(rF, rF);
        double drho = ddiv(fabs(dsub(rF, rC)), dadd(fabs(rsq), 1.0e-30));
        double dv = ddiv(fabs(dsub(vF, vC)), dadd(fabs(vF), 1.0e-30));
        if (drho < tol_r && dv < tol_v) {
            if (out_type == 0) { rho_o = rC; v_o = vC; t_o = tC; }
            else if (out_type == 1) { rho_o = rF; v_o = vF; t_o = tF; }
            else {
                double rr = dsub(dmul(4.0, rF), dmul(3.0, rC));
                double vr = dsub(dmul(4.0, vF), dmul(3.0, vC));
                double tr = dsub(dmul(4.0, tF), dmul(3.0, tC));
                if (rr < 0.0) rr = 0.0;
                rho_o = rr; v_o = vr; t_o = tr;
            }
            return k;
        }
        if (!(isfinite(rF) && isfinite(vF))) break;
        rC = rF; vC = vF; tC = tF;
    }
    // after the loop N = 2^nlev = 2 * N_last
    micro_lc(rho, v, t, 4 * N + 1, hg, gn, l2, rho_o, v_o, t_o);
    return -1;
}

// Adaptive full Levi-Civita step, nsphere.c:2231-2334.  Entries are spread so
// that consecutive particles land on different warps: each is a long serial
// chain, and one per warp keeps lanes from waiting on one another.
__global__ void __launch_bounds__(128) k_levi_civita(StepArgs a)
{
    const unsigned cnt = a.ctr->lc_count;
    if (cnt == 0) return;
    const double Mpt = a.ctr->point_mass;
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    for (int64_t e = (int64_t)lane * warps + gw; e < cnt; e += 32 * warps) {
        uint32_t i = a.lc_idx[e];
        double r_in = a.r_in[i], v_in = a.v_in[i], ell = a.ell[i];
        double gn = gnum_of(i, a.n, a.G, a.M, Mpt);
        int lvmax = 0;
        double ro = r_in, vo = v_in;
        if (!(r_in < 1.0e-30)) {
            double l2 = dmul(ell, ell);
            double rho = sqrt(r_in);
            double v = v_in, t = 0.0;
            double dtau;
            if (r_in > 1.0e-30 && a.N_taumin > 0)
                dtau = ddiv(a.dt, dmul(dmul(2.0, r_in), (double)a.N_taumin));
            else
                dtau = ddiv(a.dt, 100.0);
            int64_t steps = 0;
            bool done = false;
            for (;;) {
                if (t >= a.dt) break;
                double rn, vn, tn;
                int lv = tau_step_lc(rho, v, t, dtau, a.tol_r, a.tol_v, a.nlev, gn, l2,
                                     a.out_type, rn, vn, tn);
                if (lv < 0) lvmax = -1;
                else if (lvmax >= 0 && lv > lvmax) lvmax = lv;
                if (tn > a.dt) {
                    double alpha = 0.0;
                    if (fabs(dsub(tn, t)) > 1.0e-30) alpha = ddiv(dsub(a.dt, t), dsub(tn, t));
                    double rf = dadd(rho, dmul(alpha, dsub(rn, rho)));
                    double vf = dadd(v, dmul(alpha, dsub(vn, v)));
                    ro = dmul(rf, rf);
                    vo = vf;
                    done = true;
                    break;
                }
                rho = rn; v = vn; t = tn;
                steps++;
                if (steps > a.max_tau_steps || !(isfinite(rho) && isfinite(t))) {
                    atomicOr(&a.ctr->status, NSG_ST_TAU_CAP);
                    break;
                }
            }
            if (!done) { ro = dmul(rho, rho); vo = v; }
        }
        a.r_out[i] = ro;
        a.v_out[i] = vo;
        a.level[i] = (int8_t)(lvmax < 0 ? kLevelLcFallback : kLevelLcBase + lvmax);
    }
}

// ------------------------------------------------------------ fixed-step KDK

// First half of the method-2 body (nsphere.c:5487-5505): kick with the rank of the
// current order, then drift.
__global__ void __launch_bounds__(256)
k_kick_drift(double *__restrict__ r, double *__restrict__ v, const double *__restrict__ a0,
             int64_t n, double dt)
{
    // a0 is gnum_i/r^2 + ell^2/r^3 at the current radius and rank: the force the
    // reference recomputes for this kick (same operands, same result).
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double vi = dadd(v[i], dmul(dmul(0.5, a0[i]), dt));
        v[i] = vi;
        r[i] = dadd(r[i], dmul(vi, dt));
    }
}

static StepArgs make_args(nsg_ctx *c)
{
    // the fused pass reads copy `src` through c->perm and writes copy `dst`
    StepArgs a{};
    const int src = c->cur, s = 1 - c->cur;
    a.r_in = c->r[s]; a.v_in = c->vr[s]; a.ell = c->ell[s]; a.a0 = c->a0;
    a.r_out = c->r[s]; a.v_out = c->vr[s];
    a.ell_out = c->ell[s]; a.aux_out = c->aux[s]; a.id_out = c->id[s]; a.inv = c->inv;
    a.perm = c->perm;
    a.r_src = c->r[src]; a.v_src = c->vr[src]; a.l_src = c->ell[src]; a.aux_src = c->aux[src];
    a.id_src = c->id[src];
    a.level = c->level;
    a.n = c->n;
    a.G = c->p.G; a.M = c->p.M_total; a.dt = c->p.dt;
    a.tol_r = c->p.tol_r; a.tol_v = c->p.tol_v;
    a.max_subdiv = c->p.max_subdiv;
    int nlev = 0;
    for (int64_t N = 1; N <= c->p.max_subdiv && nlev < kMaxLevels - 1; N *= 2) nlev++;
    a.nlev = nlev;
    const double h = c->p.dt;
    a.hk_c0 = h / (2.0 * 1.0);
    a.ms_c0 = h / (1.0 * 1.0);
    for (int k = 0; k < kMaxLevels; k++) {
        const double N = (double)((int64_t)1 << (k < 62 ? k : 62));
        a.hk_f[k] = h / (4.0 * N);
        a.ms_f[k] = h / (2.0 * N);
    }
    a.out_type = c->p.out_type;
    a.method = c->p.method;
    a.lc_rule = c->p.lc_rule;
    a.lc_alpha = c->p.lc_alpha;
    a.lc_radius = c->p.lc_radius;
    a.N_taumin = c->p.N_taumin;
    a.max_tau_steps = c->p.max_tau_steps;
    a.ctr = c->ctr;
    for (int b = 0; b < 2; b++) { a.q_idx[b] = c->q_idx[b]; a.q_r[b] = c->q_r[b]; a.q_v[b] = c->q_v[b]; }
    a.lc_idx = c->lc_idx;
    return a;
}

int integrate_adaptive(nsg_ctx *c)
{
    if (int rc = sort_perm(c)) return rc;
    StepArgs a = make_args(c);
    cudaStream_t s = c->stream;
    cudaError_t e;
    // reset queue counters (qcount[] and lc_count live at the head of DevCounters)
    e = cudaMemsetAsync(&c->ctr->lc_count, 0, sizeof(unsigned) * (kMaxLevels + 2), s);
    if (e != cudaSuccess) return cuda_err(c, e, "memset queue counters");
    const int grid = grid_for(c, c->n, 256, 8);
    {
        // algorithmic bytes: perm 4, gather r v ell id 28, write r v ell id 28, inv 4, level 1
        ProfScope ps(c, "gather_level0", (double)c->n * (4 + 28 + 28 + 4 + 1 + (c->p.carry_aux ? 16 : 0)));
        if (c->p.carry_aux) k_gather_level0<true><<<grid, 256, 0, s>>>(a);
        else k_gather_level0<false><<<grid, 256, 0, s>>>(a);
        c->launches += 1;
    }
    c->cur = 1 - c->cur;
    c->inv_valid = true;
    c->sorted = false;  // radii moved
    if (c->p.method == NSG_METHOD_ADAPTIVE_LC && c->p.lc_rule != NSG_LC_OFF) {
        e = cudaEventRecord(c->ev_fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
        if (e != cudaSuccess) return cuda_err(c, e, "fork side stream");
        k_levi_civita<<<c->num_sms * 4, 128, 0, c->side>>>(a);
        c->launches += 1;
        e = cudaEventRecord(c->ev_join, c->side);
        if (e != cudaSuccess) return cuda_err(c, e, "join record");
    }
    {
        ProfScope ps(c, "leap_levels", 0.0);
        for (int k = 1; k < a.nlev; k++) k_level<<<c->num_sms * 8, 256, 0, s>>>(a, k);
        c->launches += a.nlev - 1;
    }
    if (c->p.method == NSG_METHOD_ADAPTIVE_LC && c->p.lc_rule != NSG_LC_OFF) {
        e = cudaStreamWaitEvent(s, c->ev_join, 0);
        if (e != cudaSuccess) return cuda_err(c, e, "join wait");
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, "integrator kernels");
    return NSG_OK;
}

int kdk_first_half(nsg_ctx *c)
{
    const int s = c->cur;
    ProfScope ps(c, "kdk_kick_drift", (double)c->n * (24 + 16));
    k_kick_drift<<<grid_for(c, c->n, 256), 256, 0, c->stream>>>(c->r[s], c->vr[s], c->a0, c->n, c->p.dt);
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "kick_drift");
}

}  // namespace nsg
