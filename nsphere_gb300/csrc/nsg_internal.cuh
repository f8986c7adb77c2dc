// nsg_internal.cuh -- shared declarations of libnsg (context, buffers, device math).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <cstring>
#include <string>
#include <vector>

#include "nsg.h"
#include "nsg_div.cuh"
#include "nsg_mul.cuh"

namespace nsg {

constexpr int kMaxLevels = 64;        // adaptive levels N = 2^k, k < 64
constexpr int kStatBins = 66;         // level histogram bins held on device
constexpr int kLcEarlyCap = 4096;     // particles below the Levi-Civita radius listed before the sort
constexpr int kLevelNotConverged = -1;
constexpr int kLevelLcBase = 100;     // Levi-Civita particles record 100 + level
constexpr int kLevelLcFallback = 99;
constexpr int kRadixBits = 8;
constexpr int kRadixBuckets = 1 << kRadixBits;
constexpr int kRadixThreads = 256;
constexpr int kRadixItems = 16;       // keys per thread per tile
constexpr int kRadixTile = kRadixThreads * kRadixItems;
constexpr int kReduceBlocks = 1024;   // fixed block count of energy partial sums
constexpr int kBucketCap = 6144;      // entries one bucket block sorts (1024 threads x 6)
constexpr int kFusedCapMax = 4096;    // entries one fused sort block holds (512 threads x 8)

// Launch shapes chosen by the autotuner (nsg_tune.cu); defaults measured on GB300.
struct Tune {
    int gl0_threads = 256;   // k_gather_level0 block size
    int gl0_bps = 8;         // k_gather_level0 blocks per SM
    int bshift = 10;         // near-sorted sort: 2^bshift sorted positions per splitter
    int lanes_bps = 4;       // k_levels_lanes blocks per SM
};

// Device-resident counters and flags of one context (a single allocation).
struct DevCounters {
    unsigned int status;                    // NSG_ST_* bits
    unsigned int lc_count;                  // particles routed to Levi-Civita
    unsigned int qcount[kMaxLevels + 1];    // queue length per leapfrog level
    unsigned int lc_next;                   // next Levi-Civita list entry a block takes
    unsigned int lc_cand;                   // particles below the Levi-Civita radius (list before the sort)
    unsigned int lc_early_ok;               // 1: the Levi-Civita list was made before the sort
    unsigned long long level_hist[kStatBins];
    double energy[2];                       // K, W of the last sort
    double point_mass;                      // current central point mass
    unsigned int need_fallback;             // 1: the radix sort must run this sort
    unsigned int pad;
};

struct MlpDev;   // nsg_mlp.cu
struct SnapWriter;   // nsg_io.cu
struct TrackDev;     // nsg_track.cu

struct KernelStat {
    std::string name;
    int64_t launches = 0;
    double total_ms = 0.0;
    double bytes = 0.0;
};

}  // namespace nsg

struct nsg_ctx {
    nsg_params p{};
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;     // leapfrog kernels beside the Levi-Civita chains
    cudaStream_t body = nullptr;     // captures the bodies of conditional graph nodes
    bool cond_nodes = false;         // the driver builds conditional graph nodes
    bool gate_fallback = false;      // eager step of a synchronous call: read the fallback flag on the host
    // the learned schedule's predictions are for the state of epoch pred_epoch; every
    // change of the resident state (upload, sort, step) starts a new epoch
    int64_t state_epoch = 0, pred_epoch = -1;
    bool g_pred_refresh = false;     // the captured steps end with the next step's predictions
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_lcsel = nullptr, ev_pre = nullptr, ev_scat = nullptr;
    bool own_stream = false;
    int device = 0;
    int num_sms = 0;
    int lc_smem = 0;                 // dynamic shared memory of a Levi-Civita block
    std::string err;

    int64_t n = 0, cap = 0;
    bool sorted = false;             // state is in (r, id) order with gnum/a0 valid
    bool inv_valid = false;          // inv maps ids to the current array order
    int64_t steps_done = 0;
    int64_t launches = 0;            // kernels launched by steps/sorts (for reporting)

    // state, two copies (sort source/destination)
    double *r[2] = {nullptr, nullptr}, *vr[2] = {nullptr, nullptr}, *ell[2] = {nullptr, nullptr};
    double *aux[2] = {nullptr, nullptr};
    int32_t *id[2] = {nullptr, nullptr};
    int cur = 0;                     // index of the live copy

    double *a0 = nullptr;            // dv/dt at the step start, per sorted position
    int32_t *inv = nullptr;          // id -> current index (the reference's inverse_map)
    int8_t *level = nullptr;         // accepted level per particle

    // radix sort scratch
    uint64_t *keys[2] = {nullptr, nullptr};
    uint32_t *vals[2] = {nullptr, nullptr};
    uint32_t *tile_counts = nullptr; // [256][ntiles]
    uint32_t *digit_tot = nullptr;   // [256]
    uint32_t *perm = nullptr;        // result of sort_perm: source index per sorted position

    nsg::Tune tune;

    // ensemble of halos (one segment for a single halo)
    int nseg = 1;
    std::vector<int64_t> h_seg_start;   // [nseg + 1]
    int64_t *d_seg_start = nullptr;
    int32_t *d_bbase = nullptr;         // [nseg + 1] first bucket of each halo
    int64_t nb_total = 0;               // buckets over all halos
    int64_t nb_cap = 0;
    double *seg_energy = nullptr;       // [2 * nseg] K, W per halo

    // near-sorted bucket sort (nsg_bucket.cu)
    uint64_t *split = nullptr;       // [nb_total] splitter keys from the last sort
    bool split_valid = false;
    unsigned int *bcnt = nullptr;    // [2 nb + 2]: counts [nb] (two-kernel path), look-back words (fused)
    unsigned int *boff = nullptr;    // [nb] bucket starts (two-kernel path)
    uint64_t *bkey = nullptr, *bpay = nullptr;      // [nb * bucket_cap] (two-kernel path)
    int64_t bslot_cap = 0;                          // entries allocated in bkey, bpay
    uint32_t *bidx = nullptr;                       // [nb * fused_cap] (fused path)
    int64_t bidx_cap = 0;                           // entries allocated in bidx

    // leapfrog level queues (ping-pong) and the Levi-Civita list
    uint32_t *q_idx[2] = {nullptr, nullptr};
    double *q_r[2] = {nullptr, nullptr}, *q_v[2] = {nullptr, nullptr};
    uint32_t *lc_idx = nullptr;
    unsigned char *lc_early = nullptr;   // [kLcEarlyCap] candidate keys, ids, sources; list sources

    double *red_part = nullptr;      // [2][kReduceBlocks] energy partials
    nsg::DevCounters *ctr = nullptr; // device counters
    nsg::DevCounters *h_ctr = nullptr; // pinned mirror

    // staging for uploads of ids given as doubles
    double *stage_d = nullptr;

    // snapshot stream (nsg_io.cu), open between nsg_snapshot_open and _close
    nsg::SnapWriter *snap = nullptr;

    // per-step trajectory recorder (nsg_track.cu), open between nsg_track_open and _close
    nsg::TrackDev *track = nullptr;

    // learned level scheduler (nsg_mlp.cu)
    nsg::MlpDev *mlp = nullptr;
    bool mlp_collect = false;        // record (features, level) of each step

    // CUDA graph of two consecutive steps, captured from the stream and replayed
    cudaGraphExec_t gexec = nullptr;
    int64_t g_launches = 0;          // kernels in one replay
    bool g_sorted = false;           // host state the graph was captured from
    bool g_failed = false;           // capture not possible here: launch eagerly

    bool profiling = false;
    std::vector<nsg::KernelStat> stats;
    std::vector<cudaEvent_t> ev_pool;
};

namespace nsg {

// ---------------------------------------------------------------- device math
// All integrator arithmetic uses explicit round-to-nearest intrinsics so that no
// multiply-add is contracted: each operation rounds like the reference's C code
// compiled with -ffp-contract=off.
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }

// Predicates and exact conversions on the integer pipe.  On GB300 every FP64
// instruction -- a comparison or an int-to-double conversion included -- occupies the
// FP64 pipe, which the throughput kernels saturate, so they test bit patterns instead.
// The bit pattern comes out of an asm move, opaque to the compiler: given the plain
// reinterpretation, it turns the masked integer compare of abs_lt back into a
// floating-point compare, with a wrong answer for NaN (true for |NaN| < y).
__device__ __forceinline__ long long dbits(double x)
{
    long long b;
    asm("mov.b64 %0, %1;" : "=l"(b) : "d"(x));
    return b;
}
// isfinite(x)
__device__ __forceinline__ bool finite_bits(double x) { return ((dbits(x) >> 52) & 0x7ff) != 0x7ff; }
// fabs(x) for a number (a NaN comes out with its sign cleared; fabs keeps it on GB300)
__device__ __forceinline__ double iabs(double x) { return __longlong_as_double(dbits(x) & 0x7fffffffffffffffll); }
// |x| < y for y not NaN (signed-integer order of the bit patterns is the order of
// non-negative doubles, and a negative y sorts below every |x|)
__device__ __forceinline__ bool abs_lt(double x, double y) { return (dbits(x) & 0x7fffffffffffffffll) < dbits(y); }
// lo < r < hi for lo >= +0 and hi not NaN; false for a NaN r, as the floating-point test
__device__ __forceinline__ bool open_between(double r, double lo, double hi)
{
    const long long b = dbits(r);
    return b > dbits(lo) && b < dbits(hi);
}
// Rare operand paths behind calls.  A branch whose other side issues FP64
// instructions is if-converted by the compiler -- both sides are computed and one is
// selected -- so an inline slow path costs its FP64 issue slots on every call; a call
// cannot be predicated that way, so its instructions run only when it is taken.  The
// operands cross the call as bit patterns (a double argument costs an FP64-pipe
// instruction at every call site, taken or not).
static __device__ __noinline__ double dmul_call_bits(unsigned long long a, unsigned long long b)
{
    return __dmul_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b));
}
static __device__ __noinline__ double dadd_call_bits(unsigned long long a, unsigned long long b)
{
    return __dadd_rn(__longlong_as_double((long long)a), __longlong_as_double((long long)b));
}
__device__ __forceinline__ double dmul_call(double a, double b)
{
    return dmul_call_bits((unsigned long long)dbits(a), (unsigned long long)dbits(b));
}
__device__ __forceinline__ double dadd_call(double a, double b)
{
    return dadd_call_bits((unsigned long long)dbits(a), (unsigned long long)dbits(b));
}

// x + 1e-30 for x >= +0 or NaN.  From x = 2^-46 up, 1e-30 is below half an ulp of x
// (2^-99), so the sum rounds to x; only smaller x take the FP64 addition.
__device__ __forceinline__ double add_1em30(double x)
{
    if (dbits(x) >= (977ll << 52)) return x;
    return dadd_call(x, 1.0e-30);
}
// 4 x: for a normal x whose product stays normal the exponent field rises by two
// (exact, as the multiplication); other x take the FP64 multiplication.
__device__ __forceinline__ double mul4(double x)
{
    const long long b = dbits(x);
    if (((unsigned)(b >> 52) & 0x7ffu) - 1u < 2044u) return __longlong_as_double(b + (2ll << 52));
    return dmul_call(4.0, x);
}
// RN(x / y) < tol, decided without the division.  RN is monotonic, and the quotient
// of two doubles is never halfway between two doubles (that would take a 54-bit odd
// significand), so RN(x/y) < tol exactly when x/y lies below the midpoint between
// tol and its predecessor: B 2^(e_t - 1076) with B = 2 m_t - 1, or B = 2^54 - 1 at
// 2^(e_t - 1077) when tol is a power of two (m_t, e_t: significand and biased
// exponent of tol).  With x = m_x 2^(e_x - 1075) and y = m_y 2^(e_y - 1075) that is
// m_x 2^D < B m_y for D = e_x - e_y + doff: true for D <= 52 (left side below
// 2^105), false for D >= 55 (left side at least 2^107), and one 64 x 64-bit product
// for D = 53, 54.
struct RatioBound {
    uint64_t B;
    int32_t doff;
    int32_t ok;   // tol is a positive normal number
};

__host__ __device__ inline RatioBound ratio_bound(double tol)
{
    uint64_t b;
    memcpy(&b, &tol, 8);
    const uint32_t et = (uint32_t)(b >> 52) & 0x7ffu;
    if ((b >> 63) != 0 || et == 0u || et == 0x7ffu) return RatioBound{0, 0, 0};
    const uint64_t mt = (b & 0x000fffffffffffffull) | (1ull << 52);
    if (mt == (1ull << 52)) return RatioBound{(1ull << 54) - 1ull, 1077 - (int32_t)et, 1};
    return RatioBound{2ull * mt - 1ull, 1076 - (int32_t)et, 1};
}

// x >= +0 or NaN, y > 0 or NaN.  `decided` is false unless tol is a positive normal,
// y is normal and x is +0 or normal; the caller then divides.
__device__ __forceinline__ bool ratio_lt(double x, double y, const RatioBound &t, bool &decided)
{
    const long long bx = dbits(x), by = dbits(y);
    const unsigned ex = (unsigned)(bx >> 52) & 0x7ffu, ey = (unsigned)(by >> 52) & 0x7ffu;
    decided = t.ok && (ey - 1u < 2046u) && (bx == 0 || ex - 1u < 2046u);
    if (bx == 0) return true;
    const int D = (int)ex - (int)ey + t.doff;
    if (D <= 52) return true;
    if (D >= 55) return false;
    const uint64_t mx = ((uint64_t)bx & 0x000fffffffffffffull) | (1ull << 52);
    const uint64_t my = ((uint64_t)by & 0x000fffffffffffffull) | (1ull << 52);
    const uint64_t rlo = t.B * my, rhi = __umul64hi(t.B, my);
    const uint64_t llo = mx << D, lhi = mx >> (64 - D);
    return lhi < rhi || (lhi == rhi && llo < rlo);
}

// x as a double, exactly, for 0 <= x < 2^32
__device__ __forceinline__ double u32_to_double(uint32_t x)
{
    if (x == 0u) return 0.0;
    const int e = 31 - __clz((int)x);
    const unsigned long long m = ((unsigned long long)x << (52 - e)) & 0x000fffffffffffffull;
    return __longlong_as_double((long long)((((unsigned long long)(1023 + e)) << 52) | m));
}

// Division: throughput-bound kernels divide on the integer/FP32 pipes (div_rn:
// the latency form with the FP64 pipe's division behind a call, nsg_div.cuh); the
// Levi-Civita chains use div_rn_lat directly and redo a tau-step on the FP64 pipe
// when it declines an operand.  All are IEEE round-to-nearest, so the choice never
// changes a result bit.
template <bool HW>
__device__ __forceinline__ double ddivx(double a, double b) { return HW ? div_rn_hw(a, b) : div_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return div_rn(a, b); }

// -(G) * (i / n) * M (+ the point-mass term when present), nsphere.c:513.  With
// G = M = 1 (the units of the benchmark halos) both products are exact: the result
// is the quotient with its sign flipped, and no FP64 instruction is issued (the
// tests of G, M and Mpt compare bit patterns on the integer pipe).
static __device__ __noinline__ double gnum_general(unsigned long long qb, unsigned long long Gb, unsigned long long Mb,
                                                   unsigned long long Mptb)
{
    const double q = __longlong_as_double((long long)qb), G = __longlong_as_double((long long)Gb);
    const double M = __longlong_as_double((long long)Mb), Mpt = __longlong_as_double((long long)Mptb);
    double g = __dmul_rn(__dmul_rn(-G, q), M);
    if (Mpt != 0.0) g = __dsub_rn(g, __dmul_rn(G, Mpt));
    return g;
}

template <bool HW = false>
__device__ __forceinline__ double gnum_of(int64_t i, int64_t n, double G, double M, double Mpt)
{
    const double q = ddivx<HW>(u32_to_double((uint32_t)i), u32_to_double((uint32_t)n));
    constexpr long long kOne = 0x3ff0000000000000ll;
    if (dbits(G) == kOne && dbits(M) == kOne && (dbits(Mpt) << 1) == 0)   // Mpt == 0.0
        return __longlong_as_double(dbits(q) ^ (long long)0x8000000000000000ull);
    return gnum_general((unsigned long long)dbits(q), (unsigned long long)dbits(G), (unsigned long long)dbits(M),
                        (unsigned long long)dbits(Mpt));
}

// 0.5 x: for a normal x whose half stays normal the exponent field falls by one
// (exact, as the multiplication); other x take the FP64 multiplication.
__device__ __forceinline__ double half_exact(double x)
{
    const long long b = dbits(x);
    if (((unsigned)(b >> 52) & 0x7ffu) - 2u < 2045u) return __longlong_as_double(b - (1ll << 52));
    return dmul_call(0.5, x);
}

// Multiplication of the throughput kernels: EM = on the integer pipes (mul_rn,
// nsg_mul.cuh), else on the FP64 pipe.  Both are IEEE round-to-nearest, so the choice
// never changes a bit; kernels bound by the FP64 pipe move their products off it,
// serial chains (bound by latency) keep the FP64 pipe's.
template <bool EM>
__device__ __forceinline__ double tmul(double a, double b) { return EM ? mul_rn(a, b) : dmul(a, b); }

// gravity + centrifugal: gnum/(r*r) + l2/(r*r*r), nsphere.c:502-535.
template <bool HW = false, bool EM = false>
__device__ __forceinline__ double acc_leap(double r, double gnum, double l2)
{
    double r2 = tmul<EM>(r, r);
    return dadd(ddivx<HW>(gnum, r2), ddivx<HW>(l2, tmul<EM>(r2, r)));
}

// Order-preserving map of a double to uint64: -0.0 -> +0.0, NaN -> all ones.
__device__ __forceinline__ uint64_t radius_key(double r)
{
    unsigned long long u = (unsigned long long)dbits(r);
    if ((u & 0x7fffffffffffffffull) > 0x7ff0000000000000ull) return ~0ull;   // NaN
    if ((u << 1) == 0ull) u = 0ull;                                           // -0 -> +0
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// Segment table of an ensemble of independent halos: halo h occupies the positions
// [start[h], start[h+1]) in every copy of the state and is sorted and integrated on
// its own (its rank and particle count enter the force, nsphere.c:513).  A single
// halo is the one-segment case.  bbase[h] is the first near-sorted bucket of halo h.
struct Seg {
    const int64_t *start;   // [nseg + 1]
    const int32_t *bbase;   // [nseg + 1]
    int nseg;
    int bshift;             // log2 of the sorted positions per splitter (bucket target)
};

struct Local {
    int64_t i, n;   // rank within the halo, halo size
    int h;          // halo
};

__device__ __forceinline__ int seg_of(const Seg &s, int64_t p)
{
    if (s.nseg <= 1) return 0;
    int lo = 0, hi = s.nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (s.start[mid] <= p) lo = mid; else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ Local local_of(const Seg &s, int64_t p, int64_t n_total)
{
    if (s.nseg <= 1) return Local{p, n_total, 0};
    const int h = seg_of(s, p);
    const int64_t st = s.start[h];
    return Local{p - st, s.start[h + 1] - st, h};
}

// Splitter of the next near-sorted sort: key(r) at every 2^bshift-th sorted
// position of each halo, written by the passes that consume a sort (from the sorted
// start-of-step radii); the first splitter of a halo is the smallest key.
__device__ __forceinline__ void write_splitter(uint64_t *S, const Seg &sg, const Local &L, double r)
{
    if ((L.i & ((1ll << sg.bshift) - 1)) == 0)
        S[sg.bbase[L.h] + (L.i >> sg.bshift)] = (L.i == 0) ? 0ull : radius_key(r);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Appends one entry per active predicate to a queue; returns the slot or -1.
__device__ __forceinline__ int warp_append(bool pred, unsigned int *counter)
{
    unsigned active = __activemask();
    unsigned mask = __ballot_sync(active, pred);
    if (!pred) return -1;
    int leader = __ffs(mask) - 1;
    unsigned base = 0;
    int lane = threadIdx.x & 31;
    if (lane == leader) base = atomicAdd(counter, (unsigned)__popc(mask));
    base = __shfl_sync(mask, base, leader);
    return (int)(base + __popc(mask & lanemask_lt()));
}

// ------------------------------------------------------------- host helpers
int set_err(nsg_ctx *c, int code, const std::string &msg);
int cuda_err(nsg_ctx *c, cudaError_t e, const char *what);
int grid_for(nsg_ctx *c, int64_t n, int threads, int per_sm = 8);

// Profiling: brackets a launch group with events when profiling is on.
struct ProfScope {
    nsg_ctx *c;
    const char *name;
    double bytes;
    cudaStream_t st;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    ProfScope(nsg_ctx *c_, const char *name_, double bytes_, cudaStream_t stream = nullptr);
    ~ProfScope();
};
void prof_flush(nsg_ctx *c);

// kernels' host launchers (return NSG_OK or error)
int sort_perm(nsg_ctx *c);                            // radix sort of the live copy -> c->perm
int sort_state(nsg_ctx *c);                           // sort_perm + gather with rank force (a0)
int sort_state_kick(nsg_ctx *c);                      // same, plus the second half-kick (KDK)
int integrate_adaptive(nsg_ctx *c);                   // method 3 / 5: sort_perm, then fused gather + levels
int kdk_first_half(nsg_ctx *c);                       // kick (a0 of the current rank) + drift
int compute_energy(nsg_ctx *c);                       // K, W of the sorted live copy
int bucket_sort_perm(nsg_ctx *c);                     // near-sorted fast path (sets need_fallback)
int fused_cap(const nsg_ctx *c);                      // entries of a fused sort block (0: fused path off)
int bucket_cap(const nsg_ctx *c);                     // slots per bucket of the two-kernel path
// scatter indices and counts for the fused kernels; with lc_thr > 0 also lists the
// Levi-Civita candidates (radius key below lc_thr) into the early-list arrays
int bucket_fused_prepare(nsg_ctx *c, cudaStream_t s, uint64_t lc_thr = 0);
bool use_fused(const nsg_ctx *c);                     // the sort of this step runs inside its consumer
// Launches the radix sort and then `tail` on stream s so that they run only when
// need_fallback is set: in a captured step as the body of a conditional graph node,
// otherwise eagerly with kernels that return at once (tail receives the flag to test).
int radix_fallback(nsg_ctx *c, cudaStream_t s, int (*tail)(nsg_ctx *, cudaStream_t, const unsigned *, void *),
                   void *arg);
inline Seg seg_table(const nsg_ctx *c) { return Seg{c->d_seg_start, c->d_bbase, c->nseg, c->tune.bshift}; }
void drop_graph(nsg_ctx *c);                          // forget the captured step graph
int set_halos(nsg_ctx *c, const int64_t *seg_n, int nseg);  // halo table + bucket layout
int begin_upload(nsg_ctx *c, int64_t n);              // size the buffers for a one-halo state
int finish_upload_ids(nsg_ctx *c);                    // ids staged as doubles -> int32, validated
void build_inv(nsg_ctx *c);                           // inv from the current id order
void snap_close(nsg_ctx *c);                          // end a snapshot stream (nsg_io.cu)
int track_step(nsg_ctx *c);                           // record the tracked particles (nsg_track.cu)
void track_free(nsg_ctx *c);
int post_psi_sorted(nsg_ctx *c, const double *r, const double *v, const double *l, int64_t n, double *psi,
                    double *E, double *tile, double *total);  // Psi_A of a sorted state (nsg_post.cu)
int64_t post_tiles(int64_t n);                           // scratch doubles post_psi_sorted needs
// predicted level per source index of the state in buffer buf (rows below *skip, when
// given, are neither read nor predicted: class 0)
int mlp_predict_state(nsg_ctx *c, const int8_t **pred, cudaStream_t st, int buf, const unsigned *skip = nullptr);
int mlp_features_state(nsg_ctx *c, cudaStream_t st);   // features of the step's start state (training set)
const int8_t *mlp_pred_buffer(nsg_ctx *c);             // the predictions' buffer (by source index)
bool learned_refresh(const nsg_ctx *c);                // learned steps predict for the next step at their end
int mlp_append_levels(nsg_ctx *c);                    // append (features, accepted level)
void mlp_free(nsg_ctx *c);
int bucket_setup(nsg_ctx *c);
int fused_force_setup(nsg_ctx *c);   // shared-memory attributes of the fused sort kernels
int fused_level0_setup(nsg_ctx *c);
int lc_setup(nsg_ctx *c);            // Levi-Civita kernel attributes
int lc_probe_substep(double *cycles_split, double *cycles_zero_gravity, double *cycles_dual);
int launch_gather(nsg_ctx *c, const int32_t *d_ids, int k, double *d_out, int32_t *d_rank);
int launch_level_hist(nsg_ctx *c);
int launch_ids_from_double(nsg_ctx *c, const double *d_src, int32_t *d_dst, int64_t n);
int launch_validate_ids(nsg_ctx *c, const int32_t *d_id, int64_t n, int *ok);

}  // namespace nsg
