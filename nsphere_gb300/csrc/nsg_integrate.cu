// nsg_integrate.cu -- per-particle integrators of the step, on the sorted state.
//
// Adaptive leapfrog (nsphere.c:1550-1735).  The reference tries N = 1, 2, 4, ...
// and returns at the first N whose coarse (2N+1 substeps) and fine (4N+1
// substeps) passes agree.  Three facts let the GPU reorganise that loop while
// returning bit-identical results:
//   * every level restarts from the step's initial (r, v) (nsphere.c:1673-1684),
//     so levels are independent of one another;
//   * the coarse pass of level k (N' = 2^k: halfKick h/(2N'), midStep h/N',
//     N' pairs) performs exactly the operations of the fine pass of level k-1
//     (N = 2^(k-1): halfKick h/(4N), midStep h/(2N), 2N pairs), so each level
//     needs only its own fine pass;
//   * every pass starts with the same half-kick at r_in, so the first force is
//     computed once.
// Work split:
//   k_gather_level0  fused with the sort's gather: level 0 for every particle
//                    (throughput-bound; divisions on the integer pipe);
//   k_levels_lanes   particles that failed level 0: a group of lanes per
//                    particle, lane j computing the fine pass of level j+1 at the
//                    same time; the group stops at the first level that agrees
//                    with the level below (latency-bound; the latency-form
//                    division, two per force in one lane without FP64 issue slots).
// Adaptive Levi-Civita (nsphere.c:1990-2334): one warp per particle, started on a
// side stream right after the sort, overlapped with the leapfrog work.  Within a
// tau-step the lanes compute the coarse N=1 pass, the fine pass of every level and
// the non-converged fallback pass at once; the first converging level decides.
// The force at the end of one substep is the force at the start of the next
// (nsphere.c:2014 and :2022 evaluate forceLCfun at the same rho), so it is
// evaluated once.
#include <cstring>

#include "nsg_fused.cuh"

namespace nsg {

constexpr uint32_t kFreshBit = 0x80000000u;   // queue entry that skipped level 0

struct StepArgs {
    // sorted copy: k_gather_level0 writes it; final (r, v) land in r_out / v_out
    double *r_out, *v_out, *ell_out, *aux_out;
    int32_t *id_out, *inv;
    double *a0;                 // start acceleration, written for queued particles only
    uint64_t *split;            // splitters of the next near-sorted sort
    // unsorted source copy and the permutation from the sort
    const uint32_t *perm;
    const double *r_src, *v_src, *l_src, *aux_src;
    const int32_t *id_src;
    int8_t *level;
    int64_t n;
    double G, M, dt, tol_r, tol_v;
    RatioBound rb_r, rb_v;      // the tolerances' midpoints below (ratio_lt)
    int nlev;                   // number of levels: floor(log2(max_subdiv)) + 1
    int out_type;
    int method;
    int lc_rule;
    double lc_alpha, lc_radius;
    int N_taumin;
    int64_t max_tau_steps;
    int nf_stop;                // a non-finite pass ends the climb / the tau-steps (nonfinite_stop)
    DevCounters *ctr;
    uint32_t *q_idx;            // particles that left level 0 (kFreshBit: skipped it)
    double *q_r, *q_v;          // their fine N=1 result (the coarse pass of level 1)
    uint32_t *lc_idx;
    const uint32_t *lc_src;     // source index of each list entry when listed before the sort, or null
    const int8_t *pred;         // learned schedule: predicted level per source index, or null
    Seg seg;                    // halos of an ensemble (ranks and sizes are per halo)
    const unsigned *run_if;     // consumers of the radix fallback: return at once unless *run_if
    uint32_t *perm_w;           // fused path: source index of each Levi-Civita particle's position
    // Substep sizes of each pass, identical for every particle, computed once on
    // the host with the same IEEE divisions as nsphere.c:1566-1577 (exact here:
    // h divided by powers of two): coarse N=1 halfKick h/2, midStep h;
    // fine N=2^k halfKick h/(4N), midStep h/(2N).
    double hk_c0, ms_c0;
    double hk_f[kMaxLevels], ms_f[kMaxLevels];
};

// Micro leapfrog, nsphere.c:1550-1607: half-kick, (pairs-1) drift-kick pairs, drift,
// half-kick.  pairs = N (coarse, 2N+1 substeps) or 2N (fine, 4N+1 substeps); the
// first acceleration a_first = acc(r_in) is passed in.
template <bool HW, bool EM = false>
__device__ __forceinline__ void micro_leap(double r, double v, double l2, double gn,
                                           double hk, double ms, int64_t pairs, double a_first,
                                           double &r_out, double &v_out)
{
    v = dadd(v, tmul<EM>(hk, a_first));
    for (int64_t pp = 1; pp <= pairs - 1; pp++) {
        r = dadd(r, tmul<EM>(ms, v));
        v = dadd(v, tmul<EM>(ms, acc_leap<HW, EM>(r, gn, l2)));
    }
    r = dadd(r, tmul<EM>(ms, v));
    v = dadd(v, tmul<EM>(hk, acc_leap<HW, EM>(r, gn, l2)));
    r_out = r;
    v_out = v;
}

// Acceptance test of nsphere.c:1688-1691 (and :2125-2128, whose radius term is
// scaled by rF^2 instead of rF).
// The quotients are only compared with the tolerances, so ratio_lt decides each test
// from the operands' bits; the division runs for the operands it leaves undecided.
template <bool HW>
__device__ __forceinline__ bool converged(double rc, double vc, double rf, double vf,
                                          double rscale, const StepArgs &a)
{
    const double xr = iabs(dsub(rf, rc)), yr = add_1em30(iabs(rscale));
    const double xv = iabs(dsub(vf, vc)), yv = add_1em30(iabs(vf));
    bool dec_r, dec_v;
    bool ok_r = ratio_lt(xr, yr, a.rb_r, dec_r);
    bool ok_v = ratio_lt(xv, yv, a.rb_v, dec_v);
    // dr, dv >= +0 or NaN; the tolerances are numbers
    if (!dec_r) ok_r = abs_lt(ddivx<HW>(xr, yr), a.tol_r);
    if (!dec_v) ok_v = abs_lt(ddivx<HW>(xv, yv), a.tol_v);
    return ok_r && ok_v;
}

template <bool EM = false>
__device__ __forceinline__ void select_out(int out_type, double rc, double vc, double rf,
                                           double vf, double &ro, double &vo)
{
    if (out_type == 0) { ro = rc; vo = vc; }
    else if (out_type == 1) { ro = rf; vo = vf; }
    else {
        ro = dsub(mul4(rf), tmul<EM>(3.0, rc));
        vo = dsub(mul4(vf), tmul<EM>(3.0, vc));
    }
}

// Routing of nsphere.c:5804-5822 (alpha rule), or a fixed radius.
__device__ __forceinline__ bool route_lc(const StepArgs &a, const Local &L, double r, double ell)
{
    if ((a.method != NSG_METHOD_ADAPTIVE_LC && a.method != NSG_METHOD_FULL_LC) || a.lc_rule == NSG_LC_OFF)
        return false;
    if (a.lc_rule == NSG_LC_RADIUS) return open_between(r, 1.0e-30, a.lc_radius);
    double r_crit = 0.0;
    if (a.method == NSG_METHOD_FULL_LC) {
        // method 4 (nsphere.c:5696-5707): M_i = (i/N) M for every rank, any ell != 0
        if (ell != 0.0) {
            const double gravPart = dmul(a.G, dmul(ddiv(u32_to_double((uint32_t)L.i), u32_to_double((uint32_t)L.n)), a.M));
            r_crit = ddiv(dmul(dmul(ell, ell), a.lc_alpha), gravPart);
        }
        return (r > 1.0e-30) && (r < r_crit);
    }
    if (fabs(ell) > 1.0e-30) {
        double M_enc;
        if (L.i == 0) M_enc = dmul(dmul(0.1, ddiv(1.0, u32_to_double((uint32_t)L.n))), a.M);
        else M_enc = dmul(ddiv(u32_to_double((uint32_t)L.i), u32_to_double((uint32_t)L.n)), a.M);
        double gravPart = dmul(a.G, M_enc);
        r_crit = ddiv(dmul(dmul(ell, ell), a.lc_alpha), gravPart);
    }
    return (r > 1.0e-30) && (r < r_crit);
}

// Level-0 work of sorted position i (rank L within its halo) for the particle
// (r, v, ell, idv) taken from source index s: write it into sorted order, write the
// inverse map (nsphere.c:5789-5794) and the next sort's splitter, then -- unless it is
// routed to Levi-Civita (nsphere.c:5804-5822), which another kernel handles --
// compute its rank force numerator and start acceleration (nsphere.c:502-535) and
// run adaptive level 0.  FUSED: the caller sorted in the block (no permutation
// array), so a Levi-Civita particle leaves its source index in perm_w for the
// chains, and joins their list here when it was not made before the sort.
template <bool AUX, bool FUSED>
__device__ __forceinline__ void level0_particle(const StepArgs &a, int64_t i, const Local &L, uint32_t s,
                                                double r, double v, double ell, int32_t idv, double Mpt,
                                                bool last)
{
    a.ell_out[i] = ell;
    a.id_out[i] = idv;
    if (AUX) a.aux_out[i] = a.aux_src[s];
    a.inv[idv] = (int32_t)i;
    write_splitter(a.split, a.seg, L, r);
    if (route_lc(a, L, r, ell)) {
        if (FUSED) {
            a.perm_w[i] = s;
            if (!a.ctr->lc_early_ok) {
                const int slot = warp_append(true, &a.ctr->lc_count);
                a.lc_idx[slot] = (uint32_t)i;
            }
        }
        return;
    }
    // The pass is bound by the FP64 pipe, and the integer pipes already carry its
    // divisions and the sort: the coarse pass's, ell^2's and the Richardson step's
    // multiplications (8 of 19) run on the integer pipes, the rest on the FP64 pipe
    // (all 19 on the integer pipes measured slower than none).
    constexpr bool EM = true;
    const double gn = gnum_of(L.i, L.n, a.G, a.M, Mpt);
    const double l2 = tmul<EM>(ell, ell);
    const double af = acc_leap(r, gn, l2);
    // learned schedule: a particle predicted to need level >= 1 goes straight to
    // the level-parallel kernel, which tests every level from 0 upward
    const bool fresh = (a.pred != nullptr) && !last && a.pred[s] >= 1;
    double rc = 0.0, vc = 0.0, rf = 0.0, vf = 0.0;
    bool done = false;
    if (!fresh) {
        micro_leap<false, EM>(r, v, l2, gn, a.hk_c0, a.ms_c0, 1, af, rc, vc);
        micro_leap<false>(r, v, l2, gn, a.hk_f[0], a.ms_f[0], 2, af, rf, vf);
        const bool ok = converged<false>(rc, vc, rf, vf, rf, a);
        const bool bad = !(finite_bits(rf) && finite_bits(vf));
        done = ok || last || (bad && a.nf_stop);
        if (done) {
            double ro, vo;
            select_out<EM>(a.out_type, rc, vc, rf, vf, ro, vo);
            a.r_out[i] = ro;
            a.v_out[i] = vo;
            a.level[i] = ok ? 0 : kLevelNotConverged;
            if (!ok) atomicOr(&a.ctr->status, bad ? (NSG_ST_NAN | NSG_ST_NOT_CONVERGED) : NSG_ST_NOT_CONVERGED);
        }
    }
    const int q = warp_append(!done, &a.ctr->qcount[1]);
    if (!done) {
        a.r_out[i] = r;          // start values for the higher levels
        a.v_out[i] = v;
        a.a0[i] = af;
        a.q_idx[q] = fresh ? ((uint32_t)i | kFreshBit) : (uint32_t)i;
        a.q_r[q] = rf;
        a.q_v[q] = vf;
    }
}

// Fused pass after the sort, per sorted position i: gather the particle into
// sorted order through the permutation and do its level-0 work.  The pass is
// FP64-bound, so the gather traffic hides under the arithmetic.
template <bool AUX>
__global__ void __launch_bounds__(512) k_gather_level0(StepArgs a)
{
    if (a.run_if && *a.run_if == 0u) return;   // fallback consumer: the fused kernel did the work
    const double Mpt = a.ctr->point_mass;
    const bool last = (a.nlev <= 1);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = a.perm[i];
        const double r = a.r_src[s], v = a.v_src[s], ell = a.l_src[s];
        const int32_t idv = a.id_src[s];
        level0_particle<AUX, false>(a, i, local_of(a.seg, i, a.n), s, r, v, ell, idv, Mpt, last);
    }
}

// The same with the near-sorted sort done in the block (nsg_fused.cuh): block b sorts
// bucket b and does the level-0 work of its sorted positions off[b] ..; the sort's
// integer and shared-memory work overlaps other blocks' FP64 work on the same SM.
template <bool AUX, int T>
__global__ void __launch_bounds__(T, T == 128 ? 6 : (T == 256 ? 4 : 1)) k_fused_level0(StepArgs a, FusedSort fs)
{
    const unsigned over = *fs.over;
    if (blockIdx.x == 0 && threadIdx.x == 0) a.ctr->need_fallback = over;   // read after this kernel
    if (over) return;
    const int b = blockIdx.x;
    const uint32_t m = fused_count(fs, b);
    if (m == 0u) {
        fused_lookback_empty<T>(fs, b);
        return;
    }
    extern __shared__ __align__(16) unsigned char fsm[];
    uint64_t *sr, *sv;
    const int64_t base = fused_bucket_sort<T>(fs, b, m, a.r_src, a.id_src, fsm, sr, sv);
    const double Mpt = a.ctr->point_mass;
    const bool last = (a.nlev <= 1);
    const int h = halo_of_bucket(a.seg, b);
    const int64_t hs = a.seg.nseg <= 1 ? 0 : a.seg.start[h];
    const int64_t hn = a.seg.nseg <= 1 ? a.n : a.seg.start[h + 1] - hs;
    for (uint32_t j = threadIdx.x; j < m; j += T) {
        const int64_t i = base + j;
        const uint64_t e = sv[j];
        const uint32_t s = (uint32_t)e;
        const double r = entry_radius(sr[j], e, a.r_src);
        const double v = a.v_src[s], ell = a.l_src[s];
        level0_particle<AUX, true>(a, i, Local{i - hs, hn, h}, s, r, v, ell, entry_id(e), Mpt, last);
    }
}

// Particles that leave level 0.  A group of G lanes (a power of two) serves one
// particle and every lane runs one pass of it at the same time:
//   plain layout (FULL = false; the particle failed level 0, whose fine pass is
//     queued): lane j runs the fine pass of level j+1, G >= nlev-1;
//   full layout (learned schedule; some particles skipped level 0): lane 0 runs
//     the coarse N=1 pass, lane j >= 1 the fine pass of level j-1, G >= nlev+1.
// All lanes advance one drift-kick pair per iteration, so the fine pass of level L
// ends at iteration 2^(L+1); the test of level L then compares it with the pass
// below it, levels in the reference's order, and the group stops at the first
// level that passes (or the last level).
template <bool FULL>
__global__ void __launch_bounds__(256) k_levels_lanes(StepArgs a, int G)
{
    const unsigned cnt = a.ctr->qcount[1];
    if (cnt == 0) return;
    const double Mpt = a.ctr->point_mass;
    const int lane = threadIdx.x & 31;
    const int j = lane & (G - 1);              // pass of this lane within its group
    const int g0 = lane & ~(G - 1);            // first lane of the group
    const int groups_per_warp = 32 / G;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    const int nl = a.nlev - 1;                 // highest level
    int64_t pairs = 0;
    double hk = 0.0, ms = 0.0;
    if (FULL) {
        if (j == 0) { pairs = 1; hk = a.hk_c0; ms = a.ms_c0; }
        else if (j <= a.nlev) { pairs = (int64_t)1 << j; hk = a.hk_f[j - 1]; ms = a.ms_f[j - 1]; }
    } else if (j < nl) {
        pairs = (int64_t)2 << (j + 1); hk = a.hk_f[j + 1]; ms = a.ms_f[j + 1];
    }
    for (int64_t round = 0;; round++) {
        const int64_t e = (round * warps + gw) * groups_per_warp + (lane / G);
        if (__all_sync(0xffffffffu, e >= (int64_t)cnt)) break;
        const bool have = e < (int64_t)cnt;
        uint32_t i = 0;
        int kstart = 1;                        // first level this group tests
        double v_in = 0.0, l2 = 0.0, gn = 0.0, af = 0.0, rq = 0.0, vq = 0.0, r = 0.0;
        if (have) {
            const uint32_t raw = a.q_idx[e];
            i = raw & ~kFreshBit;
            if (raw & kFreshBit) kstart = 0;
            r = a.r_out[i];
            v_in = a.v_out[i];
            const double ell = a.ell_out[i];
            l2 = dmul(ell, ell);
            const Local L = local_of(a.seg, i, a.n);
            gn = gnum_of(L.i, L.n, a.G, a.M, Mpt);
            af = a.a0[i];
            rq = a.q_r[e];
            vq = a.q_v[e];
        }
        bool active = have;                    // the group is still searching
        double v = dadd(v_in, dmul(hk, af));
        double rf = 0.0, vf = 0.0;             // this lane's finished pass
        int64_t it = 0;
        int kcheck = FULL ? 0 : 1;             // level tested next (same in every group)
        while (__any_sync(0xffffffffu, active)) {
            // one drift-kick pair; the last pair of a pass ends with the half-kick
            if (active && it < pairs) {
                r = dadd(r, dmul(ms, v));
                if (it + 1 < pairs) v = dadd(v, dmul(ms, acc_leap(r, gn, l2)));
                else { v = dadd(v, dmul(hk, acc_leap(r, gn, l2))); rf = r; vf = v; }
            }
            it++;
            // the fine pass of level kcheck ended at it = 2^(kcheck+1)
            if (kcheck <= nl && it == ((int64_t)2 << kcheck)) {
                const int srcF = FULL ? g0 + kcheck + 1 : g0 + kcheck - 1;
                const int srcC = FULL ? g0 + kcheck : (kcheck > 1 ? srcF - 1 : srcF);
                const double rF = __shfl_sync(0xffffffffu, rf, srcF);
                const double vF = __shfl_sync(0xffffffffu, vf, srcF);
                const double rC0 = __shfl_sync(0xffffffffu, rf, srcC);
                const double vC0 = __shfl_sync(0xffffffffu, vf, srcC);
                const double rC = (!FULL && kcheck == 1) ? rq : rC0;
                const double vC = (!FULL && kcheck == 1) ? vq : vC0;
                if (active && kcheck >= kstart) {
                    const bool ok = converged<false>(rC, vC, rF, vF, rF, a);
                    const bool bad = !(finite_bits(rF) && finite_bits(vF));
                    if (ok || (bad && a.nf_stop) || kcheck == nl) {
                        if (j == 0) {
                            double ro, vo;
                            select_out(a.out_type, rC, vC, rF, vF, ro, vo);
                            a.r_out[i] = ro;
                            a.v_out[i] = vo;
                            a.level[i] = ok ? (int8_t)kcheck : (int8_t)kLevelNotConverged;
                            if (!ok) atomicOr(&a.ctr->status, bad ? (NSG_ST_NAN | NSG_ST_NOT_CONVERGED)
                                                                  : NSG_ST_NOT_CONVERGED);
                        }
                        active = false;
                    }
                }
                kcheck++;
            }
        }
    }
}

// ---------------------------------------------------------- Levi-Civita path

// Lists the Levi-Civita particles of the sorted order (the routing of
// k_gather_level0); runs on the side stream right after the sort.
__global__ void __launch_bounds__(256) k_lc_select(StepArgs a)
{
    if (a.run_if && *a.run_if == 0u) return;   // fallback consumer: the fused kernel listed them
    if (a.ctr->lc_early_ok) return;   // listed before the sort (k_lc_early_rank)
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < a.n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t s = a.perm[i];
        const bool lc = route_lc(a, local_of(a.seg, i, a.n), a.r_src[s], a.l_src[s]);
        const int slot = warp_append(lc, &a.ctr->lc_count);
        if (lc) a.lc_idx[slot] = (uint32_t)i;
    }
}

// Levi-Civita list before the sort (fixed-radius rule, one halo).  Every particle
// whose sort key is below the key of lc_radius precedes all others in the sorted
// order, so its sorted position is its rank among those particles: they are listed
// here (one pass over the radii), ranked by k_lc_early_rank, and the Levi-Civita
// chains start while the sort runs.  More than kLcEarlyCap of them leave
// lc_early_ok at 0, and k_lc_select makes the list after the sort instead.
__global__ void __launch_bounds__(256) k_lc_early_collect(StepArgs a, uint64_t kthr, uint64_t *__restrict__ ckey,
                                                          int32_t *__restrict__ cid, uint32_t *__restrict__ csrc)
{
    for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < a.n;
         s += (int64_t)gridDim.x * blockDim.x) {
        const uint64_t k = radius_key(a.r_src[s]);
        const bool cand = k < kthr;
        const int slot = warp_append(cand, &a.ctr->lc_cand);
        if (cand && slot < kLcEarlyCap) {
            ckey[slot] = k;
            cid[slot] = a.id_src[s];
            csrc[slot] = (uint32_t)s;
        }
    }
}

// Ranks the candidates by (key, id) -- the sort's order -- and lists the Levi-Civita
// ones with their sorted position and source index.  One block.
constexpr size_t kLcRankSmem = (size_t)kLcEarlyCap * (8 + 4 + 4);

__global__ void __launch_bounds__(1024) k_lc_early_rank(StepArgs a, const uint64_t *__restrict__ ckey,
                                                        const int32_t *__restrict__ cid,
                                                        const uint32_t *__restrict__ csrc, uint32_t *__restrict__ lsrc)
{
    extern __shared__ __align__(16) unsigned char rk_sm[];
    uint64_t *sk = reinterpret_cast<uint64_t *>(rk_sm);
    int32_t *si = reinterpret_cast<int32_t *>(rk_sm + (size_t)kLcEarlyCap * 8);
    int32_t *sh = reinterpret_cast<int32_t *>(rk_sm + (size_t)kLcEarlyCap * 12);
    const unsigned cnt = a.ctr->lc_cand;
    if (cnt > (unsigned)kLcEarlyCap) return;
    // halos are contiguous in the unsorted state as in the sorted one: a candidate's
    // halo follows from its source index
    for (unsigned e = threadIdx.x; e < cnt; e += blockDim.x) {
        sk[e] = ckey[e];
        si[e] = cid[e];
        sh[e] = seg_of(a.seg, (int64_t)csrc[e]);
    }
    __syncthreads();
    for (unsigned e = threadIdx.x; e < cnt; e += blockDim.x) {
        const uint64_t k = sk[e];
        const int32_t id = si[e];
        const int32_t h = sh[e];
        unsigned rank = 0;   // (r, id) rank within the halo: every particle below is a candidate
        for (unsigned j = 0; j < cnt; j++)
            rank += (sh[j] == h && (sk[j] < k || (sk[j] == k && si[j] < id))) ? 1u : 0u;
        const uint32_t s = csrc[e];
        const int64_t st = a.seg.nseg <= 1 ? 0 : a.seg.start[h];
        const int64_t nh = a.seg.nseg <= 1 ? a.n : a.seg.start[h + 1] - st;
        if (route_lc(a, Local{(int64_t)rank, nh, h}, a.r_src[s], a.l_src[s])) {
            const unsigned slot = atomicAdd(&a.ctr->lc_count, 1u);
            a.lc_idx[slot] = (uint32_t)(st + rank);
            lsrc[slot] = s;
        }
    }
    if (threadIdx.x == 0) a.ctr->lc_early_ok = 1u;
}

// Division in the Levi-Civita chains.  FAST: the latency-oriented division, with
// `bad` recording whether any quotient must be redone on the FP64 pipe; otherwise
// the FP64 pipe's division (zero dividends answered directly).
template <bool FAST>
__device__ __forceinline__ double lc_div(double a, double b, bool &bad)
{
    if (FAST) {
        bool ok;
        const double q = div_rn_lat(a, b, ok);
        bad |= !ok;
        return q;
    }
    return div_rn_hw(a, b);
}

// Levi-Civita force gnum/(rho*rho) + l2/(rho*rho*rho*rho), nsphere.c:563-599,
// 1777-1787, with the division above.  ZG (a zero gravity numerator, the innermost
// particle without a central mass): gnum/(rho*rho) is a signed zero and adding it
// returns l2/rho^4 unchanged, since that quotient is never -0 (l2 >= 0, rho^4 >= 0)
// and every quotient the fast division accepts is finite.
// SPLIT (lanes 16-31 mirror lanes 0-15): the lower lane of each pair divides l2 by
// rho^4 and the upper one gnum by rho^2 in the same instructions, and the quotients
// are exchanged -- one division's latency instead of two that the warp would issue
// in turn.  Both lanes then add the same operands in the same order.
template <bool FAST, bool ZG = false, bool SPLIT = false>
__device__ __forceinline__ double lc_force(double rho, double gn, double l2, bool &bad)
{
    const double p2 = dmul(rho, rho);
    const double p4 = dmul(dmul(p2, rho), rho);
    if (FAST && ZG) return lc_div<FAST>(l2, p4, bad);
    if (FAST && SPLIT) {
        const bool hi = (threadIdx.x & 16) != 0;
        const double q = lc_div<FAST>(hi ? gn : l2, hi ? p2 : p4, bad);
        const double qo = __shfl_xor_sync(0xffffffffu, q, 16);
        return dadd(q, qo);   // IEEE addition commutes: both halves get gravity + centrifugal
    }
    // both quotients in every lane: the gravity one as soon as rho^2 is known, so
    // that it runs while rho^4 is formed
    const double qg = lc_div<FAST>(gn, p2, bad);
    return dadd(qg, lc_div<FAST>(l2, p4, bad));
}

struct LcTau {
    double r, v, t;   // end of the tau-step (rho, v, physical time; t only when computed inline)
    int lv;           // accepted level, -1: fallback or non-finite
    int lc, lf;       // lanes whose times make the end time (-1: not needed)
};

// Exact x/2 for normal x with a biased exponent above 1; other operands set `bad`.
__device__ __forceinline__ double lc_half(double x, bool &bad)
{
    const uint64_t u = (uint64_t)__double_as_longlong(x);
    const uint32_t ex = (uint32_t)(u >> 52) & 0x7ffu;
    bad |= (ex - 2u) >= 2045u;
    return __longlong_as_double((long long)(u - (1ull << 52)));
}

// Acceptance test of nsphere.c:2125-2128 with the chain's division.
template <bool FAST>
__device__ __forceinline__ bool lc_converged(double rc, double vc, double rf, double vf, double rscale,
                                             double tol_r, double tol_v, bool &bad)
{
    const double dr = lc_div<FAST>(iabs(dsub(rf, rc)), dadd(iabs(rscale), 1.0e-30), bad);
    const double dv = lc_div<FAST>(iabs(dsub(vf, vc)), dadd(iabs(vf), 1.0e-30), bad);
    return abs_lt(dr, tol_r) && abs_lt(dv, tol_v);
}

// Slots of each lane's pass in a tau-step record of radii (PAIR form): lane 0 the
// coarse pass (3 substeps), lane 1+k the fine pass of level k, lane nlev+1 the
// fallback pass.
__host__ __device__ __forceinline__ int64_t lc_slot(int lane, int nlev)
{
    if (lane == 0) return 0;
    const int k = lane - 1;                      // 3 + sum_{j<k} (4*2^j + 1)
    return 3 + 4 * (((int64_t)1 << k) - 1) + k;
}
__host__ __device__ __forceinline__ int64_t lc_slots(int nlev)
{
    return lc_slot(nlev + 1, nlev) + 4 * ((int64_t)1 << nlev) + 1;
}

// One adaptive tau-step from (rho, v, t) (nsphere.c:2077-2186), every lane running
// its own pass: lane 0 the coarse N=1 pass (3 substeps), lane 1+k the fine pass of
// level k (4*2^k+1 substeps; it is also the coarse pass of level k+1), lane nlev+1
// the fallback fine pass at N = 2^nlev.  Level k is decided as soon as its fine pass
// ends.  The loop is bounded by the fallback pass (fb_sub substeps) whatever the
// values.  hdt*force is carried from one substep to the next: the reference forms
// the same product at the end of a substep and at the start of the next.
// PAIR: the physical time is left to a companion warp; each lane stores the radius
// after each of its substeps at xs[ss] (its own slots), and the result names the
// lanes whose times the end time is made of.  A tau-step run past the particle's
// end is abandoned at the next level check once `abandon` is set (lv = -3).
template <bool FAST, bool PAIR, bool ZG, typename IT, bool SPLIT = PAIR>
__device__ __forceinline__ LcTau lc_tau_step(const StepArgs &a, double rho, double v, double t,
                                             double gn, double l2, double dtau, double hdt,
                                             IT my_sub, IT fb_sub, int nlev, double *xs,
                                             const volatile int *abandon, bool &bad)
{
    double pr = rho, pv = v, pt = t, fr = rho, fv = v;
    double hpf = dmul(hdt, lc_force<FAST, ZG, SPLIT>(rho, gn, l2, bad));
    LcTau o{rho, v, t, -2, -1, -1};
    int kcheck = 0;
    IT next_end = 5;                     // substeps after which level kcheck's fine pass ends
    for (IT ss = 0; o.lv == -2; ss++) {
        // every lane computes (the warp issues each instruction once whatever the
        // active lanes); the working registers of a lane whose pass has ended run on
        // unused, and the pass's final state is kept aside (fr, fv), so that no select
        // sits on the dependent chain
        const bool act = ss < my_sub;
        bool bs = false;
        const double vh = dadd(pv, hpf);
        const double hp = (FAST && PAIR) ? lc_half(pr, bs) : dmul(0.5, pr);
        const double rnx = dadd(pr, dmul(dtau, dmul(hp, vh)));
        const double hf2 = dmul(hdt, lc_force<FAST, ZG, SPLIT>(rnx, gn, l2, bs));
        const double vnx = dadd(vh, hf2);
        if (PAIR) {
            if (act && (threadIdx.x & 16) == 0) xs[ss] = rnx;
        } else {
            const double rm = dmul(0.5, dadd(pr, rnx));
            const double ptn = dadd(pt, dmul(dtau, dmul(rm, rm)));
            pt = act ? ptn : pt;
        }
        if (ss + 1 == my_sub) {
            fr = rnx;
            fv = vnx;
        }
        pr = rnx;
        pv = vnx;
        hpf = hf2;
        bad |= act && bs;
        if (kcheck < nlev && ss + 1 == next_end) {
            if (PAIR) {
                // the companion warp has ended the particle: this tau-step is not needed
                const int ab = __shfl_sync(0xffffffffu, (threadIdx.x & 31) == 0 ? *abandon : 0, 0);
                if (ab) { o.lv = -3; break; }
            }
            const int lf = 1 + kcheck, lcz = kcheck;  // fine(k) lane, coarse(k) lane
            const double rF = __shfl_sync(0xffffffffu, fr, lf);
            const double vF = __shfl_sync(0xffffffffu, fv, lf);
            const double rC = __shfl_sync(0xffffffffu, fr, lcz);
            const double vC = __shfl_sync(0xffffffffu, fv, lcz);
            double tF = 0.0, tC = 0.0;
            if (!PAIR) {
                tF = __shfl_sync(0xffffffffu, pt, lf);
                tC = __shfl_sync(0xffffffffu, pt, lcz);
            }
            const double rsq = dmul(rF, rF);
            if (lc_converged<FAST>(rC, vC, rF, vF, rsq, a.tol_r, a.tol_v, bad)) {
                if (a.out_type == 0) { o.r = rC; o.v = vC; o.t = tC; o.lc = lcz; }
                else if (a.out_type == 1) { o.r = rF; o.v = vF; o.t = tF; o.lf = lf; }
                else {
                    double rr = dsub(dmul(4.0, rF), dmul(3.0, rC));
                    o.v = dsub(dmul(4.0, vF), dmul(3.0, vC));
                    if (!PAIR) o.t = dsub(dmul(4.0, tF), dmul(3.0, tC));
                    if (rr < 0.0) rr = 0.0;
                    o.r = rr;
                    o.lc = lcz;
                    o.lf = lf;
                }
                o.lv = kcheck;
            } else if (a.nf_stop && !(isfinite(rF) && isfinite(vF))) {
                o.r = rF; o.v = vF; o.t = tF;   // non-finite: stop climbing
                o.lf = lf;
                o.lv = -1;
            }
            kcheck++;
            next_end = 4 * ((int64_t)1 << kcheck) + 1;
        }
        if (o.lv == -2 && kcheck >= nlev && ss + 1 == fb_sub) {
            o.r = __shfl_sync(0xffffffffu, fr, nlev + 1);
            o.v = __shfl_sync(0xffffffffu, fv, nlev + 1);
            if (!PAIR) o.t = __shfl_sync(0xffffffffu, pt, nlev + 1);
            o.lf = nlev + 1;
            o.lv = -1;
        }
    }
    return o;
}

// One warp per Levi-Civita particle (nsphere.c:2231-2334), tau-steps until the
// physical time passes dt.  Each tau-step runs first with the latency-oriented
// division; if any lane met an operand that it does not handle, the warp redoes
// that tau-step from its start with the FP64 pipe's division, so every result is
// the one the reference computes.  Requires nlev + 2 <= 32 (max_subdiv < 2^30,
// checked by the host).  Launched with one warp per block and the largest dynamic
// shared memory a block may take, which it does not use: each block then has an SM
// to itself, and the chain's FP64 instructions never queue behind other kernels'.
__global__ void __launch_bounds__(32) k_levi_civita_lanes(StepArgs a)
{
    const unsigned cnt = a.ctr->lc_count;
    if (cnt == 0) return;
    const double Mpt = a.ctr->point_mass;
    const int lane = threadIdx.x & 31;
    const int nlev = a.nlev;
    int64_t my_sub = 0;                        // substeps of this lane's pass (0: idle)
    if (lane == 0) my_sub = 3;
    else if (lane <= nlev) my_sub = 4 * ((int64_t)1 << (lane - 1)) + 1;
    else if (lane == nlev + 1) my_sub = 4 * ((int64_t)1 << nlev) + 1;
    const int64_t fb_sub = 4 * ((int64_t)1 << nlev) + 1;
    for (;;) {
        const unsigned e = __shfl_sync(0xffffffffu, lane == 0 ? atomicAdd(&a.ctr->lc_next, 1u) : 0u, 0);
        if (e >= cnt) break;
        const uint32_t i = a.lc_idx[e];
        const uint32_t s = a.lc_src ? a.lc_src[e] : a.perm[i];
        const double r_in = a.r_src[s], v_in = a.v_src[s], ell = a.l_src[s];
        const Local L = local_of(a.seg, i, a.n);
        const double gn = gnum_of<true>(L.i, L.n, a.G, a.M, Mpt);
        int lvmax = 0;
        double ro = r_in, vo = v_in;
        if (!(r_in < 1.0e-30)) {
            const double l2 = dmul(ell, ell);
            double rho = sqrt(r_in);
            double v = v_in, t = 0.0;
            double hg;
            if (r_in > 1.0e-30 && a.N_taumin > 0)
                hg = __ddiv_rn(a.dt, dmul(dmul(2.0, r_in), (double)a.N_taumin));
            else
                hg = __ddiv_rn(a.dt, 100.0);
            const double dtau = my_sub ? __ddiv_rn(hg, (double)my_sub) : 0.0;
            const double hdt = dmul(0.5, dtau);
            int64_t steps = 0;
            bool done = false;
            for (;;) {
                if (t >= a.dt) break;
                bool bad = false;
                LcTau o = lc_tau_step<true, false, false, int64_t>(a, rho, v, t, gn, l2, dtau, hdt, my_sub, fb_sub, nlev,
                                                                   nullptr, nullptr, bad);
                if (__any_sync(0xffffffffu, bad)) {
                    bool unused = false;
                    o = lc_tau_step<false, false, false, int64_t>(a, rho, v, t, gn, l2, dtau, hdt, my_sub, fb_sub, nlev,
                                                              nullptr, nullptr, unused);
                }
                if (o.lv < 0) lvmax = -1;
                else if (lvmax >= 0 && o.lv > lvmax) lvmax = o.lv;
                // ---- physical-time bookkeeping of nsphere.c:2290-2323
                if (o.t > a.dt) {
                    double alpha = 0.0;
                    if (fabs(dsub(o.t, t)) > 1.0e-30) alpha = __ddiv_rn(dsub(a.dt, t), dsub(o.t, t));
                    const double rf = dadd(rho, dmul(alpha, dsub(o.r, rho)));
                    const double vf = dadd(v, dmul(alpha, dsub(o.v, v)));
                    ro = dmul(rf, rf);
                    vo = vf;
                    done = true;
                    break;
                }
                rho = o.r; v = o.v; t = o.t;
                steps++;
                if (steps > a.max_tau_steps || (a.nf_stop && !(isfinite(rho) && isfinite(t)))) {
                    if (lane == 0) atomicOr(&a.ctr->status, NSG_ST_TAU_CAP);
                    break;
                }
            }
            if (!done) { ro = dmul(rho, rho); vo = v; }
        }
        if (lane == 0) {
            a.r_out[i] = ro;
            a.v_out[i] = vo;
            a.level[i] = (int8_t)(lvmax < 0 ? kLevelLcFallback : kLevelLcBase + lvmax);
        }
    }
}

// Named barriers of the paired kernel (barrier 0 is __syncthreads): FULL(b) after
// the leading warp wrote tau-step record b, EMPTY(b) after the trailing warp read it.
__device__ __forceinline__ void lc_bar_sync(int id) { asm volatile("bar.sync %0, 64;" ::"r"(id) : "memory"); }
__device__ __forceinline__ void lc_bar_arrive(int id) { asm volatile("bar.arrive %0, 64;" ::"r"(id) : "memory"); }
constexpr int kLcFull = 1, kLcEmpty = 3;

struct LcRecord {
    double r, v;      // end of the tau-step (rho, v)
    int lv, lc, lf;   // accepted level and the lanes whose times make the end time
    int pad;
};

// Shared memory of the paired kernel (all dynamic, so that the whole opt-in size can
// be requested): two tau-step records, the stop flag, the particle taken, the
// termination index, each lane's dtau, then two buffers of lc_slots(nlev) radii.
__host__ __device__ __forceinline__ size_t lc_pair_smem(int nlev)
{
    return 2 * sizeof(LcRecord) + 16 + 32 * sizeof(double) + 2 * (size_t)lc_slots(nlev) * sizeof(double);
}

// Levi-Civita particles with two warps each (nsphere.c:2231-2334); needs nlev + 2
// <= 16 (lanes 16-31 of the leading warp mirror lanes 0-15 for the split force).  A warp cannot
// overlap its own FP64 instructions on GB300 (each occupies it for the full 64-cycle
// latency), so the physical-time chain t += dtau (rho_mid)^2, which no decision of
// the tau-step reads, runs on a second warp.  The leading warp runs tau-steps back
// to back (lc_tau_step, PAIR form), storing each lane's radii in one of two buffers
// and publishing a record; the trailing warp replays the time sums of the lanes the
// record names, in the reference's order, and applies the time bookkeeping of
// nsphere.c:2290-2323: it decides when the particle is done, interpolates, writes
// the result and raises the stop flag.  The leading warp reads the flag before each
// tau-step from the third on, so it runs at most one tau-step past the end.
// Barrier protocol (count 64 = both warps): for m >= 2 the leader syncs on
// EMPTY(m&1) before tau-step m (the trailer is done with record m-2, whose buffer
// it reuses) and arrives at FULL(m&1) after it.  The trailer syncs on FULL(m&1),
// reads record m (or, once stopped, just consumes it) and arrives at EMPTY(m&1).
// The leader reads the stop flag after each EMPTY sync; when set, it writes
// term_at = m, arrives at FULL(m&1) without a record (the termination token) and
// syncs on EMPTY((m+1)&1) to absorb the trailer's arrival for record m-1; the
// trailer leaves when the FULL it synced on is the token.  Every barrier phase then
// has both warps (checked by a model of the two warps over random interleavings),
// so both leave together, and the leader runs at most one tau-step past the end.
__global__ void __launch_bounds__(64) k_levi_civita_pair(StepArgs a)
{
    extern __shared__ __align__(16) unsigned char lc_sm[];
    LcRecord *rec = reinterpret_cast<LcRecord *>(lc_sm);
    volatile int *stop = reinterpret_cast<volatile int *>(lc_sm + 2 * sizeof(LcRecord));
    volatile unsigned *take = reinterpret_cast<volatile unsigned *>(lc_sm + 2 * sizeof(LcRecord) + 4);
    volatile long long *term_at = reinterpret_cast<volatile long long *>(lc_sm + 2 * sizeof(LcRecord) + 8);
    double *dtau_sm = reinterpret_cast<double *>(lc_sm + 2 * sizeof(LcRecord) + 16);
    double *xbuf = dtau_sm + 32;
    const unsigned cnt = a.ctr->lc_count;
    if (cnt == 0) return;
    const double Mpt = a.ctr->point_mass;
    const int lane = threadIdx.x & 31;
    const int role = lane & 15;                // leading warp: lanes 16-31 mirror lanes 0-15
    const bool lead = threadIdx.x < 32;
    const int nlev = a.nlev;
    const int64_t W = lc_slots(nlev);
    int64_t my_sub = 0;                        // substeps of this lane's pass (0: idle)
    if (role == 0) my_sub = 3;
    else if (role <= nlev) my_sub = 4 * ((int64_t)1 << (role - 1)) + 1;
    else if (role == nlev + 1) my_sub = 4 * ((int64_t)1 << nlev) + 1;
    const int64_t fb_sub = 4 * ((int64_t)1 << nlev) + 1;
    const int64_t off = my_sub ? lc_slot(role, nlev) : 0;
    for (;;) {
        __syncthreads();                       // the previous particle's buffers are free
        if (threadIdx.x == 0) *take = atomicAdd(&a.ctr->lc_next, 1u);   // next particle of the list
        __syncthreads();
        const unsigned e = *take;
        if (e >= cnt) break;
        const uint32_t i = a.lc_idx[e];
        const uint32_t s = a.lc_src ? a.lc_src[e] : a.perm[i];
        const double r_in = a.r_src[s], v_in = a.v_src[s], ell = a.l_src[s];
        if (threadIdx.x == 0) { *stop = 0; *term_at = -1; }
        if (r_in < 1.0e-30) {
            if (threadIdx.x == 0) {
                a.r_out[i] = r_in;
                a.v_out[i] = v_in;
                a.level[i] = (int8_t)kLevelLcBase;
            }
            continue;
        }
        const double rho0 = sqrt(r_in);
        double hg;
        if (r_in > 1.0e-30 && a.N_taumin > 0)
            hg = __ddiv_rn(a.dt, dmul(dmul(2.0, r_in), (double)a.N_taumin));
        else
            hg = __ddiv_rn(a.dt, 100.0);
        const double dtau = my_sub ? __ddiv_rn(hg, (double)my_sub) : 0.0;
        if (lead && lane < 16) dtau_sm[lane] = dtau;
        __syncthreads();
        if (lead) {
            const Local L = local_of(a.seg, i, a.n);
            const double gn = gnum_of<true>(L.i, L.n, a.G, a.M, Mpt);
            const double l2 = dmul(ell, ell);
            const double hdt = dmul(0.5, dtau);
            const bool zg = (gn == 0.0);
            const int sub32 = (int)my_sub, fb32 = (int)fb_sub;   // nlev <= 10 here
            double rho = rho0, v = v_in;
            for (int64_t m = 0;; m++) {
                const int b = (int)(m & 1);
                if (m >= 2) {
                    lc_bar_sync(kLcEmpty + b);
                    const int st = __shfl_sync(0xffffffffu, lane == 0 ? *stop : 0, 0);
                    if (st) {
                        if (lane == 0) *term_at = m;
                        __threadfence_block();
                        __syncwarp();
                        lc_bar_arrive(kLcFull + b);
                        lc_bar_sync(kLcEmpty + (b ^ 1));
                        break;
                    }
                }
                double *xs = xbuf + b * W + off;
                bool bad = false;
                LcTau o = zg ? lc_tau_step<true, true, true, int>(a, rho, v, 0.0, gn, l2, dtau, hdt, sub32, fb32,
                                                                  nlev, xs, stop, bad)
                             : lc_tau_step<true, true, false, int>(a, rho, v, 0.0, gn, l2, dtau, hdt, sub32, fb32,
                                                                   nlev, xs, stop, bad);
                if (o.lv != -3 && __any_sync(0xffffffffu, bad)) {
                    bool unused = false;
                    o = lc_tau_step<false, true, false, int>(a, rho, v, 0.0, gn, l2, dtau, hdt, sub32, fb32, nlev,
                                                             xs, stop, unused);
                }
                if (lane == 0) rec[b] = LcRecord{o.r, o.v, o.lv, o.lc, o.lf, 0};
                __threadfence_block();
                __syncwarp();
                lc_bar_arrive(kLcFull + b);
                rho = o.r;
                v = o.v;
            }
        } else {
            double rho = rho0, v = v_in, t = 0.0, ro = 0.0, vo = 0.0;
            int64_t steps = 0;
            int lvmax = 0;
            bool stopped = false;
            for (int64_t m = 0;; m++) {
                const int b = (int)(m & 1);
                lc_bar_sync(kLcFull + b);
                if (*term_at == m) break;      // the leader's termination token
                if (stopped) {                 // a tau-step run past the end: discarded
                    lc_bar_arrive(kLcEmpty + b);
                    continue;
                }
                bool fin = false;
                if (t >= a.dt) {               // nsphere.c:2245: no further tau-step
                    ro = dmul(rho, rho);
                    vo = v;
                    fin = true;
                } else {
                    const LcRecord R = rec[b];
                    // time sums of the named lanes, in the reference's order
                    const int L = lane == 0 ? R.lc : (lane == 1 ? R.lf : -1);
                    double pt = t;
                    if (L >= 0) {
                        const int64_t ns = (L == 0) ? 3 : 4 * ((int64_t)1 << (L - 1)) + 1;
                        const double dl = dtau_sm[L];
                        const double *x = xbuf + b * W + lc_slot(L, nlev);
                        double pr = rho;
                        for (int64_t ss = 0; ss < ns; ss++) {
                            const double rnx = x[ss];
                            const double rm = dmul(0.5, dadd(pr, rnx));
                            pt = dadd(pt, dmul(dl, dmul(rm, rm)));
                            pr = rnx;
                        }
                    }
                    const double tC = __shfl_sync(0xffffffffu, pt, 0);
                    const double tF = __shfl_sync(0xffffffffu, pt, 1);
                    double tn;
                    if (R.lc >= 0 && R.lf >= 0) tn = dsub(dmul(4.0, tF), dmul(3.0, tC));
                    else if (R.lc >= 0) tn = tC;
                    else tn = tF;
                    if (R.lv < 0) lvmax = -1;
                    else if (lvmax >= 0 && R.lv > lvmax) lvmax = R.lv;
                    if (tn > a.dt) {
                        double alpha = 0.0;
                        if (fabs(dsub(tn, t)) > 1.0e-30) alpha = __ddiv_rn(dsub(a.dt, t), dsub(tn, t));
                        const double rf = dadd(rho, dmul(alpha, dsub(R.r, rho)));
                        const double vf = dadd(v, dmul(alpha, dsub(R.v, v)));
                        ro = dmul(rf, rf);
                        vo = vf;
                        fin = true;
                    } else {
                        rho = R.r; v = R.v; t = tn;
                        steps++;
                        if (steps > a.max_tau_steps || (a.nf_stop && !(isfinite(rho) && isfinite(t)))) {
                            if (lane == 0) atomicOr(&a.ctr->status, NSG_ST_TAU_CAP);
                            ro = dmul(rho, rho);
                            vo = v;
                            fin = true;
                        }
                    }
                }
                if (fin) {
                    stopped = true;
                    if (lane == 0) {
                        *stop = 1;
                        a.r_out[i] = ro;
                        a.v_out[i] = vo;
                        a.level[i] = (int8_t)(lvmax < 0 ? kLevelLcFallback : kLevelLcBase + lvmax);
                    }
                }
                __threadfence_block();
                __syncwarp();
                lc_bar_arrive(kLcEmpty + b);
            }
        }
    }
}

// The Levi-Civita force with every quotient exact: the latency-form divisions, and
// the FP64 pipe's when one of them does not claim its result.
__device__ __forceinline__ double lc_force_exact(double rho, double gn, double l2)
{
    bool bad = false;
    const double f = lc_force<true>(rho, gn, l2, bad);
    if (!bad) return f;
    return lc_force<false>(rho, gn, l2, bad);
}

// Method 4's fixed-dtau Levi-Civita leapfrog (doLeviCivitaLeapfrog, nsphere.c:1827-1937):
// one thread per particle, taken from the list through the atomic counter.  Each
// substep kicks, drifts rho, kicks and adds dtau rho_mid^2 to the physical time until
// it reaches dt, then interpolates (alpha = 1 when the substep added no time).  The
// force at the start of a substep is the one at the end of the previous.
__global__ void __launch_bounds__(32) k_levi_civita_fixed(StepArgs a)
{
    const unsigned cnt = a.ctr->lc_count;
    if (cnt == 0) return;
    const double Mpt = a.ctr->point_mass;
    for (;;) {
        const unsigned e = atomicAdd(&a.ctr->lc_next, 1u);
        if (e >= cnt) break;
        const uint32_t i = a.lc_idx[e];
        const uint32_t s = a.lc_src ? a.lc_src[e] : a.perm[i];
        const double r_in = a.r_src[s], v_in = a.v_src[s], ell = a.l_src[s];
        const Local L = local_of(a.seg, i, a.n);
        const double gn = gnum_of<true>(L.i, L.n, a.G, a.M, Mpt);
        const double l2 = dmul(ell, ell);
        double dtau;
        if (r_in > 1.0e-30 && a.N_taumin > 0)
            dtau = __ddiv_rn(a.dt, dmul(dmul(2.0, r_in), (double)a.N_taumin));
        else
            dtau = __ddiv_rn(a.dt, 100.0);
        const double hdt = dmul(0.5, dtau);
        double rho = sqrt(r_in), v = v_in, t = 0.0, ro = 0.0, vo = 0.0;
        double f = lc_force_exact(rho, gn, l2);
        int64_t steps = 0;
        bool done = false, capped = false;
        while (!done) {
            if (t >= a.dt) {
                ro = dmul(rho, rho);
                vo = v;
                break;
            }
            const double vh = dadd(v, dmul(hdt, f));
            const double rn = dadd(rho, dmul(dtau, dmul(dmul(0.5, rho), vh)));
            const double f2 = lc_force_exact(rn, gn, l2);
            const double vn = dadd(vh, dmul(hdt, f2));
            const double rm = dmul(0.5, dadd(rho, rn));
            const double tn = dadd(t, dmul(dtau, dmul(rm, rm)));
            if (tn >= a.dt) {
                double alpha = 1.0;
                if (fabs(dsub(tn, t)) > 1.0e-30) alpha = __ddiv_rn(dsub(a.dt, t), dsub(tn, t));
                const double rf = dadd(rho, dmul(alpha, dsub(rn, rho)));
                ro = dmul(rf, rf);
                vo = dadd(v, dmul(alpha, dsub(vn, v)));
                done = true;
            } else {
                rho = rn;
                v = vn;
                t = tn;
                f = f2;
                steps++;
                if (steps > a.max_tau_steps || (a.nf_stop && !(isfinite(rho) && isfinite(t)))) {
                    ro = dmul(rho, rho);
                    vo = v;
                    capped = true;
                    done = true;
                }
            }
        }
        if (capped) atomicOr(&a.ctr->status, NSG_ST_TAU_CAP);
        a.r_out[i] = ro;
        a.v_out[i] = vo;
        a.level[i] = (int8_t)kLevelLcBase;
    }
}

// Cycles per substep of lc_tau_step (fast form, PAIR) in a fallback tau-step that
// one warp runs alone on an SM: split force (nonzero gravity numerator) and zero
// gravity.  Synthetic inputs; the tolerance 1e-300 keeps every level from converging.
template <bool ZG, bool SPLIT>
__global__ void __launch_bounds__(32) k_lc_probe(StepArgs a, double gn, long long *cyc, double *out)
{
    __shared__ double xs[2304];
    __shared__ int abandon;
    const int lane = threadIdx.x & 31, role = lane & 15;
    if (lane == 0) abandon = 0;
    __syncwarp();
    const int nlev = a.nlev;
    int my_sub = 0;
    if (role == 0) my_sub = 3;
    else if (role <= nlev) my_sub = 4 * (1 << (role - 1)) + 1;
    else if (role == nlev + 1) my_sub = 4 * (1 << nlev) + 1;
    const int fb = 4 * (1 << nlev) + 1;
    const double dtau = my_sub ? __ddiv_rn(1.0e-3, (double)my_sub) : 0.0, hdt = dmul(0.5, dtau);
    const int64_t off = my_sub ? lc_slot(role, nlev) : 0;
    bool bad = false;
    const long long t0 = clock64();
    LcTau o = lc_tau_step<true, true, ZG, int, SPLIT>(a, 0.0156, 0.03, 0.0, gn, 5.6e-11, dtau, hdt, my_sub, fb,
                                                      nlev, xs + off, &abandon, bad);
    asm volatile("" : "+d"(o.r), "+d"(o.v));
    const long long t1 = clock64();
    out[lane] = o.r + o.v + o.lv + (bad ? 1.0 : 0.0);
    if (lane == 0) cyc[0] = t1 - t0;
}

int lc_probe_substep(double *cycles_split, double *cycles_zero_gravity, double *cycles_dual)
{
    StepArgs a;
    memset(&a, 0, sizeof(a));
    a.nlev = 8;                                  // lc_slots(8) = 2056 <= 2304
    a.tol_r = 1e-300;
    a.tol_v = 1e-300;
    a.out_type = 2;
    long long *cyc = nullptr;
    double *out = nullptr;
    cudaError_t e = cudaMalloc((void **)&cyc, sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc((void **)&out, 32 * sizeof(double));
    for (int kind = 0; kind < 3 && e == cudaSuccess; kind++) {
        for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {
            if (kind == 1) k_lc_probe<true, true><<<1, 32>>>(a, -0.0, cyc, out);
            else if (kind == 0) k_lc_probe<false, true><<<1, 32>>>(a, -2.4e-7, cyc, out);
            else k_lc_probe<false, false><<<1, 32>>>(a, -2.4e-7, cyc, out);
            e = cudaDeviceSynchronize();
        }
        long long h = 0;
        if (e == cudaSuccess) e = cudaMemcpy(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost);
        const double v = (double)h / (4 * (1 << a.nlev) + 1);
        if (kind == 1) *cycles_zero_gravity = v;
        else if (kind == 0) *cycles_split = v;
        else *cycles_dual = v;
    }
    cudaFree(cyc);
    cudaFree(out);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "levi-civita substep probe");
    return NSG_OK;
}

int lc_setup(nsg_ctx *c)
{
    int dev = 0, smem = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_levi_civita_lanes, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_levi_civita_pair, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_lc_early_rank, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLcRankSmem);
    if (e != cudaSuccess) return cuda_err(c, e, "levi-civita kernel setup");
    c->lc_smem = smem;
    return NSG_OK;
}

// ------------------------------------------------------------ fixed-step KDK

// First half of the method-2 body (nsphere.c:5487-5505): kick with the rank of the
// current order, then drift.  a0 is gnum_i/r^2 + ell^2/r^3 at the current radius
// and rank: the force the reference recomputes for this kick (same operands,
// same result).
__global__ void __launch_bounds__(256)
k_kick_drift(double *__restrict__ r, double *__restrict__ v, const double *__restrict__ a0,
             int64_t n, double dt)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        double vi = dadd(v[i], mul_rn(half_exact(a0[i]), dt));
        v[i] = vi;
        r[i] = dadd(r[i], mul_rn(vi, dt));
    }
}

static StepArgs make_args(nsg_ctx *c)
{
    // the fused pass reads copy `src` through c->perm and writes copy `dst`
    StepArgs a{};
    const int src = c->cur, dst = 1 - c->cur;
    a.r_out = c->r[dst]; a.v_out = c->vr[dst]; a.ell_out = c->ell[dst]; a.aux_out = c->aux[dst];
    a.id_out = c->id[dst]; a.inv = c->inv; a.a0 = c->a0; a.split = c->split;
    a.perm = c->perm;
    a.r_src = c->r[src]; a.v_src = c->vr[src]; a.l_src = c->ell[src]; a.aux_src = c->aux[src];
    a.id_src = c->id[src];
    a.level = c->level;
    a.n = c->n;
    a.G = c->p.G; a.M = c->p.M_total; a.dt = c->p.dt;
    a.tol_r = c->p.tol_r; a.tol_v = c->p.tol_v;
    a.rb_r = ratio_bound(a.tol_r); a.rb_v = ratio_bound(a.tol_v);
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
    a.nf_stop = c->p.nonfinite_stop != 0;
    a.ctr = c->ctr;
    a.q_idx = c->q_idx[0]; a.q_r = c->q_r[0]; a.q_v = c->q_v[0];
    a.lc_idx = c->lc_idx;
    a.lc_src = nullptr;
    a.pred = nullptr;
    a.seg = seg_table(c);
    a.run_if = nullptr;
    a.perm_w = nullptr;
    return a;
}

// Levi-Civita chains of the list in `a` on stream st: one block per SM (its shared
// memory request keeps other blocks off the SM): a warp cannot overlap its own FP64
// instructions, and another kernel's warps on the SM would queue on the same FP64
// pipe.  At most half of the SMs are taken; each block takes the next particle of
// the list when it is done (blocks past the list's end leave at once and free their
// SM).
static void launch_levi_civita(nsg_ctx *c, const StepArgs &a, cudaStream_t st)
{
    if (a.method == NSG_METHOD_FULL_LC)
        k_levi_civita_fixed<<<c->num_sms, 32, 0, st>>>(a);
    else if (a.nlev + 2 <= 16 && lc_pair_smem(a.nlev) <= (size_t)c->lc_smem)
        k_levi_civita_pair<<<c->num_sms / 2, 64, c->lc_smem, st>>>(a);
    else
        k_levi_civita_lanes<<<c->num_sms / 2, 32, c->lc_smem, st>>>(a);
    c->launches += 1;
}

static uint64_t radius_key_host(double r)
{
    if (r != r) return ~0ull;
    uint64_t u = 0;
    if (r != 0.0) memcpy(&u, &r, 8);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// Consumers of the radix fallback of a fused step (radix_fallback's tail): the
// Levi-Civita selection (when listed after the sort) and the level-0 gather, both
// through the radix permutation and gated by the fallback flag.
struct Level0Tail {
    StepArgs a;
    bool select;
};

static void launch_gather_level0(nsg_ctx *c, const StepArgs &a, cudaStream_t st, const char *name)
{
    // algorithmic bytes: perm 4, gather r v ell id 28, write r v ell id 28, inv 4, level 1
    ProfScope ps(c, name, (double)c->n * (4 + 28 + 28 + 4 + 1 + (c->p.carry_aux ? 16 : 0)), st);
    const int th = c->tune.gl0_threads, grid = grid_for(c, c->n, th, c->tune.gl0_bps);
    if (c->p.carry_aux) k_gather_level0<true><<<grid, th, 0, st>>>(a);
    else k_gather_level0<false><<<grid, th, 0, st>>>(a);
    c->launches += 1;
}

static int level0_tail(nsg_ctx *c, cudaStream_t st, const unsigned *run_if, void *arg)
{
    const Level0Tail *t = static_cast<const Level0Tail *>(arg);
    StepArgs a = t->a;
    a.perm = c->perm;
    a.run_if = run_if;
    if (t->select) {
        ProfScope ps(c, "lc_select_fallback", (double)c->n * 20, st);
        k_lc_select<<<grid_for(c, c->n, 256, 4), 256, 0, st>>>(a);
        c->launches += 1;
    }
    launch_gather_level0(c, a, st, "gather_level0_fallback");
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "level-0 fallback kernels");
}

// The fused sort + level 0 on stream st: index scatter and scan, one block per
// bucket, then the radix fallback with its two-kernel consumers.
static int fused_level0(nsg_ctx *c, StepArgs &a, cudaStream_t st, bool select, bool prepared = false)
{
    if (!prepared)
        if (int rc = bucket_fused_prepare(c, st)) return rc;
    a.perm = a.perm_w = c->vals[0];   // the radix fallback's even pass count ends in vals[0] too
    const int cap = fused_cap(c);
    const FusedSort fs = fused_sort_args(c, cap);
    {
        // algorithmic bytes: index 4, r id 12, v ell 16, write r v ell id 28, inv 4, level 1
        ProfScope ps(c, "fused_level0", (double)c->n * (4 + 12 + 16 + 28 + 4 + 1 + (c->p.carry_aux ? 16 : 0)), st);
        const int nb = (int)c->nb_total;
        const size_t sm = fused_smem_bytes(cap);
        if (cap == 4096) {
            if (c->p.carry_aux) k_fused_level0<true, 512><<<nb, 512, sm, st>>>(a, fs);
            else k_fused_level0<false, 512><<<nb, 512, sm, st>>>(a, fs);
        } else if (cap == 2048) {
            if (c->p.carry_aux) k_fused_level0<true, 256><<<nb, 256, sm, st>>>(a, fs);
            else k_fused_level0<false, 256><<<nb, 256, sm, st>>>(a, fs);
        } else {
            if (c->p.carry_aux) k_fused_level0<true, 128><<<nb, 128, sm, st>>>(a, fs);
            else k_fused_level0<false, 128><<<nb, 128, sm, st>>>(a, fs);
        }
        c->launches += 1;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, "fused level-0 kernel");
    Level0Tail t{a, select};
    return radix_fallback(c, st, level0_tail, &t);
}

int fused_level0_setup(nsg_ctx *c)
{
    cudaError_t e = cudaSuccess;
#define NSG_ATTR(AUXV, TV)                                                                   \
    if (e == cudaSuccess)                                                                    \
        e = cudaFuncSetAttribute(k_fused_level0<AUXV, TV>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                 (int)fused_smem_bytes(TV * kFusedItems));
    NSG_ATTR(false, 128) NSG_ATTR(true, 128) NSG_ATTR(false, 256) NSG_ATTR(true, 256) NSG_ATTR(false, 512)
    NSG_ATTR(true, 512)
#undef NSG_ATTR
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "fused level-0 attributes");
}

// Whether a learned step makes the next step's predictions at its end: one halo, the
// fixed-radius Levi-Civita rule (whose chains own the first lc_cand rows of the new
// order) and the fused sort.
bool learned_refresh(const nsg_ctx *c)
{
    const bool lc = ((c->p.method == NSG_METHOD_ADAPTIVE_LC || c->p.method == NSG_METHOD_FULL_LC) &&
                     c->p.lc_rule != NSG_LC_OFF);
    return lc && c->p.lc_rule == NSG_LC_RADIUS && c->nseg <= 1 && use_fused(c) && !c->mlp_collect;
}

int integrate_adaptive(nsg_ctx *c)
{
    const bool lc = ((c->p.method == NSG_METHOD_ADAPTIVE_LC || c->p.method == NSG_METHOD_FULL_LC) &&
                     c->p.lc_rule != NSG_LC_OFF);
    // fixed-radius rule: the Levi-Civita list is made before the sort
    const bool early = lc && c->p.lc_rule == NSG_LC_RADIUS;
    const bool learned = (c->p.sched == NSG_SCHED_LEARNED);
    // the sort runs inside the level-0 kernel unless something needs the permutation
    // before it: scheduler data collection (its samples pair features with levels
    // through it), or a Levi-Civita list made after the sort
    const bool fz = use_fused(c) && !c->mlp_collect && (early || !lc);
    if (!early && !fz)
        if (int rc = sort_perm(c)) return rc;
    StepArgs a = make_args(c);
    const bool learned_lv = learned && a.nlev > 1;
    // The scheduler's features come from the state as the step starts (source index
    // order, the previous sort's); its predictions are read by source index in the
    // level-0 pass.  Collection computes the same features.  A learned step of one
    // halo under the fixed-radius rule predicts for the next step at its own end,
    // beside its Levi-Civita chains (whose rows, the first lc_cand of the new order,
    // it leaves alone), so the next step starts with its predictions made.
    const bool refresh = learned_lv && learned_refresh(c);
    auto schedule = [&](cudaStream_t st) -> int {
        if (learned_lv) {
            if (c->pred_epoch == c->state_epoch) a.pred = mlp_pred_buffer(c);
            else if (int rc = mlp_predict_state(c, &a.pred, st, c->cur)) return rc;
        }
        if (c->mlp_collect)
            if (int rc = mlp_features_state(c, st)) return rc;
        return NSG_OK;
    };
    cudaStream_t s = c->stream;
    cudaError_t e;
    // reset queue counters (lc_count, qcount[], lc_next, lc_cand, lc_early_ok lead DevCounters)
    e = cudaMemsetAsync(&c->ctr->lc_count, 0, sizeof(unsigned) * (kMaxLevels + 5), s);
    if (e != cudaSuccess) return cuda_err(c, e, "memset queue counters");
    // With Levi-Civita particles, their kernel is launched on the main stream and the
    // leapfrog kernels run on the side stream after a cross-stream wait, which
    // resolves later: the Levi-Civita blocks, each of which needs a whole SM, are
    // placed before the leapfrog blocks fill the GPU.
    cudaStream_t ls = s;
    if (early) {
        // main: list + rank the particles below lc_radius, then their chains;
        // side: the sort, the leapfrog kernels.  The chains start ~the sort's
        // duration earlier than after the sort.
        uint64_t *ckey = reinterpret_cast<uint64_t *>(c->lc_early);
        int32_t *cid = reinterpret_cast<int32_t *>(c->lc_early + (size_t)kLcEarlyCap * 8);
        uint32_t *csrc = reinterpret_cast<uint32_t *>(c->lc_early + (size_t)kLcEarlyCap * 12);
        uint32_t *lsrc = reinterpret_cast<uint32_t *>(c->lc_early + (size_t)kLcEarlyCap * 16);
        {
            ProfScope ps(c, "lc_prepass", (double)c->n * 8);
            if (fz) {
                // one pass over the radii on the side stream: the index scatter, which
                // also lists the candidates below lc_radius; the main stream ranks them
                e = cudaEventRecord(c->ev_fork, s);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
                if (e != cudaSuccess) return cuda_err(c, e, "fork side stream");
                if (int rc = bucket_fused_prepare(c, c->side, radius_key_host(c->p.lc_radius))) return rc;
                e = cudaEventRecord(c->ev_scat, c->side);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_scat, 0);
                if (e != cudaSuccess) return cuda_err(c, e, "scatter event");
                if (int rc = schedule(c->side)) return rc;
            } else {
                k_lc_early_collect<<<grid_for(c, c->n, 256, 4), 256, 0, s>>>(a, radius_key_host(c->p.lc_radius),
                                                                              ckey, cid, csrc);
                c->launches += 1;
            }
            k_lc_early_rank<<<1, 1024, kLcRankSmem, s>>>(a, ckey, cid, csrc, lsrc);
            c->launches += 1;
        }
        // the side stream's consumer reads whether the list was made (lc_early_ok)
        e = cudaEventRecord(fz ? c->ev_pre : c->ev_fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, fz ? c->ev_pre : c->ev_fork, 0);
        if (e != cudaSuccess) return cuda_err(c, e, "fork side stream");
        {
            ProfScope ps(c, "levi_civita", 0.0);
            StepArgs ae = a;
            ae.lc_src = lsrc;
            launch_levi_civita(c, ae, s);
        }
        ls = c->side;
        if (fz) {
            // sort + level 0 in one kernel; it lists the Levi-Civita particles itself
            // when the list before the sort overflowed
            if (int rc = fused_level0(c, a, ls, true, true)) return rc;
        } else {
            if (int rc = schedule(c->side)) return rc;
            const cudaStream_t keep = c->stream;
            c->stream = c->side;
            const int rc = sort_perm(c);
            c->stream = keep;
            if (rc) return rc;
            a.perm = c->perm;
            ProfScope ps(c, "lc_select", (double)c->n * 20, ls);
            k_lc_select<<<grid_for(c, c->n, 256, 4), 256, 0, ls>>>(a);   // returns at once unless the list overflowed
            c->launches += 1;
        }
        e = cudaEventRecord(c->ev_lcsel, ls);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_lcsel, 0);
        if (e != cudaSuccess) return cuda_err(c, e, "levi-civita list event");
        {
            ProfScope ps(c, "lc_late", 0.0);
            launch_levi_civita(c, a, s);   // the list made after the sort; empty otherwise
        }
    } else if (lc) {
        if (int rc = schedule(s)) return rc;
        {
            ProfScope ps(c, "lc_select", (double)c->n * 20);
            k_lc_select<<<grid_for(c, c->n, 256, 4), 256, 0, s>>>(a);
            c->launches += 1;
        }
        e = cudaEventRecord(c->ev_fork, s);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
        if (e != cudaSuccess) return cuda_err(c, e, "fork side stream");
        ls = c->side;
        ProfScope ps(c, "levi_civita", 0.0);
        launch_levi_civita(c, a, s);
    } else {
        if (int rc = schedule(s)) return rc;
        if (fz)
            if (int rc = fused_level0(c, a, s, false)) return rc;
    }
    if (!fz) launch_gather_level0(c, a, ls, "gather_level0");
    if (a.nlev > 1) {
        ProfScope ps(c, "leap_levels", 0.0, ls);
        int G = 1;
        while (G < (learned_lv ? a.nlev + 1 : a.nlev - 1)) G <<= 1;
        if (learned_lv) k_levels_lanes<true><<<c->num_sms * c->tune.lanes_bps, 256, 0, ls>>>(a, G);
        else k_levels_lanes<false><<<c->num_sms * c->tune.lanes_bps, 256, 0, ls>>>(a, G);
        c->launches += 1;
    }
    if (refresh) {
        const int8_t *next = nullptr;
        if (int rc = mlp_predict_state(c, &next, ls, 1 - c->cur, &c->ctr->lc_cand)) return rc;
    }
    if (lc) {
        e = cudaEventRecord(c->ev_join, c->side);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_join, 0);
        if (e != cudaSuccess) return cuda_err(c, e, "join");
    }
    if (c->mlp_collect)
        if (int rc = mlp_append_levels(c)) return rc;
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, "integrator kernels");
    c->cur = 1 - c->cur;
    c->state_epoch++;
    if (refresh) c->pred_epoch = c->state_epoch;
    c->inv_valid = true;
    c->sorted = false;  // radii moved
    c->split_valid = true;
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
