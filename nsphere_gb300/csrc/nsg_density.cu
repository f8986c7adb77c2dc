// nsg_density.cu -- per-snapshot post-processing of nsphere.c:7060-7990 on the GPU:
// the snapshot's records become the resident state and are sorted with the library's
// own sort; then, per particle, the enclosed mass, the distribution potential Psi_A
// interpolated on the reference's adjusted knots, the energy and the smoothed density,
// packed into the two Rank-file record layouts.
//
// Kernels and what bounds them (n particles, G = 131072 grid points):
//   k_snap_to_state, k_pack_*        one pass over the records (HBM)
//   k_keep_*                         strictly increasing subsequence: count, scan, prefix (HBM)
//   k_psi_knots                      the knot adjustment is a sequential recurrence; one warp
//                                    advances 32 knots per iteration (closed form of repeated
//                                    addition inside one binade, below)
//   k_psi_interp                     binary search per particle (L2 latency)
//   k_cspline_chunks                 natural cubic spline coefficients: the tridiagonal system
//                                    is strictly diagonally dominant (diagonal = 2 x the
//                                    off-diagonal sum), so its inverse decays at least like
//                                    2^-|i-j|; each thread solves a 256-row chunk with 96 rows
//                                    of overlap on either side (truncation error < 2^-96
//                                    relative), so results equal a single sweep to rounding
//   k_conv                           the one-sided Gaussian smoothing, G x (kernel support)
//                                    multiply-adds on the FP64 pipe, tiled in shared memory
// The whole file compiles without FMA contraction, so every expression rounds as the
// oracle's sequential restatement does; the spline solve and the reductions differ
// from it only in summation order.
#include "nsg_internal.cuh"

#include <cmath>
#include <vector>

namespace nsg {

struct SnapIn {
    int32_t rank;
    float r, v, l;
};
static_assert(sizeof(SnapIn) == 16, "snapshot record");
static_assert(sizeof(nsg_rank_sorted) == 32 && sizeof(nsg_rank_unsorted) == 28, "rank records");

constexpr int64_t kGrid = 131072;        // density grid (nsphere.c:7384)
constexpr double kKnotStep = 1e-5;       // knot separation of the Psi_A interpolation (:7761)
constexpr int kKeepThreads = 256, kKeepItems = 16, kKeepTile = kKeepThreads * kKeepItems;
constexpr int kChunk = 256, kHalo = 96;  // spline chunks
constexpr int kConvT = 256;              // smoothing tile (outputs and kernel taps)
constexpr int kKnotWin = 4096;           // radii staged per window of the knot warp

__global__ void k_snap_to_state(const SnapIn *__restrict__ rec, int64_t n, double *__restrict__ r,
                                double *__restrict__ v, double *__restrict__ l, int32_t *__restrict__ id)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const SnapIn s = rec[i];
        r[i] = (s.r != s.r) ? 0.0 : (double)s.r;
        v[i] = (s.v != s.v) ? 0.0 : (double)s.v;
        l[i] = (double)s.l;
        id[i] = (int32_t)i;
    }
}

// ---------------------------------------------------------------- Psi_A knots

// knots K[0..n]: K[0] = 0, K[i] = R[i-1] unless R[i-1] <= K[i-1], then K[i-1] + 1e-5.
// One warp.  In "free" stretches a knot is its radius and the warp finds the first
// radius not above its predecessor with one ballot per 128 knots.  In a cascade, knot
// values are y, y (+) c, (y (+) c) (+) c, ...; while y stays in one binade [2^e, 2^e+1)
// with ulp u, y (+) c = y + K u with K = c/u rounded to nearest (c/u not a tie), as long
// as y + (K + 1) u < 2^(e+1).  So the bit pattern of the k-th value is bits(y) + k K and
// 128 knots are formed at once; the steps that leave the binade, a tie, y <= 0 or a
// subnormal y take one sequential addition.
// order-preserving key of a non-NaN double (-0 and +0 equal): integer compares only
__device__ __forceinline__ unsigned long long knot_key(double x)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(x);
    if ((u << 1) == 0ull) u = 0ull;
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

// Stages R[lo .. lo + kKnotWin) (zeros past n) into shared memory with asynchronous
// copies, all in flight at once.
__device__ __forceinline__ void knot_window(double *win, const double *__restrict__ R, int64_t n, int64_t lo)
{
    const int lane = threadIdx.x;
    __syncwarp();
    for (int q = lane; q < kKnotWin; q += 32) {
        const int64_t j = lo + q;
        if (j < n) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(win + q);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(R + j) : "memory");
        } else {
            win[q] = 0.0;
        }
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncwarp();
}

// Each lane handles kKnotPer consecutive knots, so one iteration advances up to
// 32 kKnotPer knots.
constexpr int kKnotPer = 4;

__global__ void __launch_bounds__(32) k_psi_knots(const double *__restrict__ R, int64_t n, double *__restrict__ K)
{
    __shared__ __align__(16) double win[kKnotWin];
    constexpr int SPAN = 32 * kKnotPer;
    const int lane = threadIdx.x;
    const unsigned full = 0xffffffffu;
    int64_t wb = -1;                 // R index of win[0]
    double y = 0.0;                  // last knot
    if (lane == 0) K[0] = 0.0;
    int64_t i = 1;                   // next knot
    bool free_mode = true;
    // binade of y for the closed form: exponent field, K = c/ulp, first bits above it
    int cur_e = -1;
    bool closed = false;
    unsigned long long Kst = 0, end = 0;
    while (i <= n) {
        const int64_t lo = i >= 2 ? i - 2 : 0;
        if (wb < 0 || lo < wb || i + SPAN > wb + kKnotWin) {
            knot_window(win, R, n, lo);
            wb = lo;
        }
        const int m0 = lane * kKnotPer;          // this lane's first offset from i
        if (free_mode) {
            // first offset m whose radius is not above its predecessor
            int mine = SPAN;
            double xs[kKnotPer];
#pragma unroll
            for (int q = 0; q < kKnotPer; q++) {
                const int64_t j = i + m0 + q;
                const bool in = j <= n;
                const double x = in ? win[j - 1 - wb] : 0.0;
                const double prev = (m0 + q == 0) ? y : win[j - 2 - wb];
                xs[q] = x;
                if (mine == SPAN && (!in || knot_key(x) <= knot_key(prev))) mine = in ? m0 + q : -(m0 + q) - 1;
            }
            // a negative mark ends the array (no trigger there)
            const bool hit = mine != SPAN;
            const unsigned b = __ballot_sync(full, hit);
            const int fl = b ? __ffs(b) - 1 : 32;
            const int mm = __shfl_sync(full, mine, fl < 32 ? fl : 0);
            const int f = fl < 32 ? (mm >= 0 ? mm : -mm - 1) : SPAN;   // offsets before f are plain radii
            const bool trig = fl < 32 && mm >= 0;
#pragma unroll
            for (int q = 0; q < kKnotPer; q++)
                if (m0 + q < f) K[i + m0 + q] = xs[q];
            if (!trig) {
                // every knot up to i + f - 1 is its radius
                const int64_t last = i + f - 1;           // last knot written (f >= 1 here)
                y = win[last - 1 - wb];
                i += f;
            } else {
                // knot i + f starts a cascade from its predecessor's value
                y = (f == 0) ? y : win[i + f - 2 - wb];
                i += f;
                free_mode = false;
            }
            continue;
        }
        const long long bits = __double_as_longlong(y);
        const int e = (int)(bits >> 52);     // negative for y < 0
        if (e != cur_e) {
            cur_e = e;
            closed = false;
            if (bits > 0 && e > 0 && e < 2047) {
                const double q = ldexp(kKnotStep, 1075 - e);    // c / ulp(y), exact
                if (q < 4503599627370496.0 && q - floor(q) != 0.5) {
                    closed = true;
                    Kst = (unsigned long long)rint(q);
                    end = (unsigned long long)(e + 1) << 52;
                }
            }
        }
        int L = 0;
        if (closed) {
            const unsigned long long ub = (unsigned long long)bits;
            if (Kst == 0ull || ub + (unsigned long long)SPAN * Kst + 1ull < end) L = SPAN;
            else if (end >= ub + 2ull) {
                const unsigned long long room = (end - 2ull - ub) / Kst;
                L = room > (unsigned long long)SPAN ? SPAN : (int)room;
            }
        }
        if (L <= 0) {
            const double x = win[i - 1 - wb];
            double knot;
            if (knot_key(x) <= knot_key(y)) {
                knot = y + kKnotStep;
            } else {
                knot = x;
                free_mode = true;
            }
            if (lane == 0) K[i] = knot;
            y = knot;
            i += 1;
            continue;
        }
        // offset m < L: the cascade value before knot i+m is bits + m K; it stops at the
        // first m whose radius is above that value (or past the end)
        int mine = SPAN;
        double xs[kKnotPer];
#pragma unroll
        for (int q = 0; q < kKnotPer; q++) {
            const int m = m0 + q;
            const int64_t j = i + m;
            const bool act = m < L;
            const bool in = act && j <= n;
            const double x = in ? win[j - 1 - wb] : 0.0;
            xs[q] = x;
            const unsigned long long ym = (unsigned long long)bits + (unsigned long long)m * Kst;
            if (mine == SPAN && act && (!in || knot_key(x) > (ym | 0x8000000000000000ull))) mine = m;
        }
        const unsigned sb = __ballot_sync(full, mine != SPAN);
        const int fl = sb ? __ffs(sb) - 1 : 32;
        const int f = fl < 32 ? __shfl_sync(full, mine, fl) : L;
#pragma unroll
        for (int q = 0; q < kKnotPer; q++) {
            const int m = m0 + q;
            if (m < f) K[i + m] = __longlong_as_double((long long)((unsigned long long)bits + (unsigned long long)(m + 1) * Kst));
        }
        if (f < L) {
            const int64_t jf = i + f;
            if (jf <= n) {
                const double xf = win[jf - 1 - wb];
                if (lane == 0) K[jf] = xf;
                y = xf;
                free_mode = true;
            }
            i = jf + 1;
        } else {
            y = __longlong_as_double((long long)((unsigned long long)bits + (unsigned long long)L * Kst));
            i += L;
        }
    }
}

// linear interpolation on strictly increasing knots kx[0..m) (NaN outside)
__global__ void k_psi_interp(const double *__restrict__ kx, const double *__restrict__ ky, int64_t m,
                             const double *__restrict__ x, const SnapIn *__restrict__ rec, int64_t n,
                             double *__restrict__ out)
{
    const double x0 = kx[0], x1 = kx[m - 1];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const double v = x ? x[t] : (double)rec[t].r;
        if (!(v >= x0 && v <= x1)) {
            out[t] = __longlong_as_double(0x7ff8000000000000ll);
            continue;
        }
        int64_t lo = 0, hi = m - 1;
        while (hi > lo + 1) {
            const int64_t mid = (lo + hi) / 2;
            if (kx[mid] > v) hi = mid;
            else lo = mid;
        }
        const double dx = kx[lo + 1] - kx[lo];
        out[t] = ky[lo] + (v - kx[lo]) / dx * (ky[lo + 1] - ky[lo]);
    }
}

__global__ void k_set_psi0(double *psiK, const double *total, double G, double dM)
{
    psiK[0] = G * dM * *total;
}

// ---------------------------------------------------------------- strictly increasing subsequence

__device__ __forceinline__ bool kept(const double *R, int64_t i)
{
    return i == 0 || R[i] > R[i - 1];
}

__global__ void __launch_bounds__(kKeepThreads) k_keep_counts(const double *__restrict__ R, int64_t n,
                                                              long long *__restrict__ cnt)
{
    __shared__ int sh[kKeepThreads / 32];
    const int64_t base = (int64_t)blockIdx.x * kKeepTile;
    int c = 0;
    for (int k = 0; k < kKeepItems; k++) {
        const int64_t i = base + k * kKeepThreads + threadIdx.x;
        if (i < n && kept(R, i)) c++;
    }
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        long long s = 0;
        for (int w = 0; w < kKeepThreads / 32; w++) s += sh[w];
        cnt[blockIdx.x] = s;
    }
}

// exclusive scan of cnt[0..m) in place, one block
__global__ void __launch_bounds__(1024) k_scan_ll(long long *cnt, int64_t m)
{
    __shared__ long long sh[1024];
    const int t = threadIdx.x;
    const int64_t per = (m + 1023) / 1024;
    const int64_t lo = t * per < m ? t * per : m, hi = lo + per < m ? lo + per : m;
    long long s = 0;
    for (int64_t j = lo; j < hi; j++) s += cnt[j];
    sh[t] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
        const long long v = t >= o ? sh[t - o] : 0;
        __syncthreads();
        sh[t] += v;
        __syncthreads();
    }
    long long run = t ? sh[t - 1] : 0;
    for (int64_t j = lo; j < hi; j++) {
        const long long v = cnt[j];
        cnt[j] = run;
        run += v;
    }
}

// I[i] = number of kept positions <= i
__global__ void __launch_bounds__(kKeepThreads) k_keep_prefix(const double *__restrict__ R, int64_t n,
                                                              const long long *__restrict__ off,
                                                              int32_t *__restrict__ I)
{
    __shared__ int sh[kKeepThreads];
    const int64_t base = (int64_t)blockIdx.x * kKeepTile + (int64_t)threadIdx.x * kKeepItems;
    int c = 0;
    for (int k = 0; k < kKeepItems; k++) {
        const int64_t i = base + k;
        if (i < n && kept(R, i)) c++;
    }
    sh[threadIdx.x] = c;
    __syncthreads();
    for (int o = 1; o < kKeepThreads; o <<= 1) {
        const int v = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
        __syncthreads();
        sh[threadIdx.x] += v;
        __syncthreads();
    }
    long long run = off[blockIdx.x] + (threadIdx.x ? sh[threadIdx.x - 1] : 0);
    for (int k = 0; k < kKeepItems; k++) {
        const int64_t i = base + k;
        if (i >= n) break;
        if (kept(R, i)) run++;
        I[i] = (int32_t)run;
    }
}

// Rd[k], Md[k] of the decimated subsequence (nsphere.c:7331-7361)
__global__ void k_decimate(const double *__restrict__ R, const int32_t *__restrict__ I, int64_t n, int64_t F,
                           int64_t D, int all, double step, double dM, double *__restrict__ Rd,
                           double *__restrict__ Md)
{
    const int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (k >= D) return;
    int64_t idx = k;
    if (!all) {
        idx = (int64_t)round((double)k * step);
        if (idx >= F) idx = F - 1;
    }
    // smallest position p with I[p] >= idx + 1
    int64_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const int64_t mid = (lo + hi) / 2;
        if (I[mid] >= idx + 1) hi = mid;
        else lo = mid + 1;
    }
    Rd[k] = R[lo];
    Md[k] = (double)(lo + 1) * dM;
}

__global__ void k_mono_check(const double *__restrict__ x, int64_t m, unsigned int *flag)
{
    for (int64_t i = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < m; i += (int64_t)gridDim.x * blockDim.x)
        if (!(x[i] > x[i - 1])) atomicOr(flag, 1u);
}

// the reference's strict-monotonicity repair, sequential (:7402-7409, :7446-7453)
__global__ void k_mono_fix(double *x, int64_t m)
{
    for (int64_t i = 1; i < m; i++)
        if (x[i] <= x[i - 1]) x[i] = x[i - 1] + 1e-12;
}

// ---------------------------------------------------------------- natural cubic spline

__device__ __forceinline__ void cs_row(const double *x, const double *y, int64_t i, double &h0, double &h1,
                                       double &diag, double &rhs)
{
    h0 = x[i] - x[i - 1];
    h1 = x[i + 1] - x[i];
    diag = 2.0 * (h0 + h1);
    rhs = 3.0 * ((y[i + 1] - y[i]) / h1 - (y[i] - y[i - 1]) / h0);
}

// c[0..m): c_i = y''_i / 2, natural ends.  Thread t owns rows [1 + t kChunk, ...).
__global__ void k_cspline_chunks(const double *__restrict__ x, const double *__restrict__ y, int64_t m,
                                 double *__restrict__ c, double *__restrict__ scratch)
{
    const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t rows = m - 2;
    if (t == 0) {
        c[0] = 0.0;
        c[m - 1] = 0.0;
    }
    if (t * kChunk >= rows) return;
    const int64_t s = 1 + t * kChunk, e = s + kChunk < m - 1 ? s + kChunk : m - 1;
    const int64_t a = s - kHalo > 1 ? s - kHalo : 1, b = e + kHalo < m - 1 ? e + kHalo : m - 1;
    double *cp = scratch + t * 2 * (kChunk + 2 * kHalo), *dp = cp + (kChunk + 2 * kHalo);
    double pc = 0.0, pd = 0.0;
    for (int64_t i = a; i < b; i++) {
        double h0, h1, diag, rhs;
        cs_row(x, y, i, h0, h1, diag, rhs);
        const double den = (i == a) ? diag : diag - h0 * pc;
        pc = h1 / den;
        pd = (i == a) ? rhs / den : (rhs - h0 * pd) / den;
        cp[i - a] = pc;
        dp[i - a] = pd;
    }
    double nx = 0.0;
    for (int64_t i = b - 1; i >= a; i--) {
        const double ci = (i == b - 1) ? dp[i - a] : dp[i - a] - cp[i - a] * nx;
        if (i >= s && i < e) c[i] = ci;
        nx = ci;
    }
}

__device__ __forceinline__ double cs_eval(const double *x, const double *y, const double *c, int64_t i, double v)
{
    const double h = x[i + 1] - x[i], dx = v - x[i];
    const double b = (y[i + 1] - y[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
    const double d = (c[i + 1] - c[i]) / (3.0 * h);
    return y[i] + dx * (b + dx * (c[i] + dx * d));
}

// b_i, d_i of every interval, the same expressions as cs_eval: the evaluation at
// many points then needs no division
__global__ void k_cs_coef(const double *__restrict__ x, const double *__restrict__ y, const double *__restrict__ c,
                          int64_t m, double *__restrict__ bo, double *__restrict__ dout)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= m - 1) return;
    const double h = x[i + 1] - x[i];
    bo[i] = (y[i + 1] - y[i]) / h - h * (c[i + 1] + 2.0 * c[i]) / 3.0;
    dout[i] = (c[i + 1] - c[i]) / (3.0 * h);
}

// largest i <= m-2 with x[i] <= v
__device__ __forceinline__ int64_t interval(const double *x, int64_t m, double v)
{
    int64_t lo = 0, hi = m - 1;
    while (hi > lo + 1) {
        const int64_t mid = (lo + hi) / 2;
        if (x[mid] > v) hi = mid;
        else lo = mid;
    }
    return lo;
}

// ---------------------------------------------------------------- density grid

__global__ void k_grid(double lmin, double dlog, double *__restrict__ lg, double *__restrict__ rg)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= kGrid) return;
    const double l = lmin + (double)i * dlog;
    lg[i] = l;
    rg[i] = pow(10.0, l);
}

__global__ void k_mass_grid(const double *__restrict__ rg, const double *__restrict__ Rd,
                            const double *__restrict__ Md, const double *__restrict__ cd, int64_t D,
                            double *__restrict__ mg)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= kGrid) return;
    const double v = rg[i];
    if (v < Rd[0]) mg[i] = Md[0];
    else if (v > Rd[D - 1]) mg[i] = Md[D - 1];
    else mg[i] = cs_eval(Rd, Md, cd, interval(Rd, D, v), v);
}

__global__ void k_dens_grid(const double *__restrict__ rg, const double *__restrict__ mg, double *__restrict__ dg,
                            unsigned int *flag)
{
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i < 1 || i >= kGrid - 1) return;
    const double dr = rg[i + 1] - rg[i - 1];
    double d;
    if (dr > 1e-15) {
        d = (mg[i + 1] - mg[i - 1]) / dr;
    } else {
        atomicOr(flag, 1u);
        d = 0.0;
    }
    dg[i] = d < 1e-10 ? 1e-10 : d;
}

// the sequential form, for grids with coincident points (:7496-7514)
__global__ void k_dens_grid_seq(const double *rg, const double *mg, double *dg)
{
    for (int64_t i = 1; i < kGrid - 1; i++) {
        const double dr = rg[i + 1] - rg[i - 1];
        double d = (dr > 1e-15) ? (mg[i + 1] - mg[i - 1]) / dr : ((i > 1) ? dg[i - 1] : 0.0);
        dg[i] = d < 1e-10 ? 1e-10 : d;
    }
}

__global__ void k_dens_ends(double *dg)
{
    dg[0] = dg[1];
    dg[kGrid - 1] = dg[kGrid - 2];
}

// unnormalised one-sided Gaussian taps and the last nonzero one
__global__ void k_gauss(double step, double sigma, double pref, double *__restrict__ kn, unsigned int *last)
{
    const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (m >= kGrid) return;
    const double x = (double)m * step;
    const double v = pref * exp(-0.5 * (x / sigma) * (x / sigma));
    kn[m] = v;
    if (v > 0.0) atomicMax(last, (unsigned int)m);
}

__global__ void __launch_bounds__(1024) k_sum_grid(const double *__restrict__ a, double *out)
{
    __shared__ double sh[32];
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < kGrid; i += 1024) s += a[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double t = sh[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (threadIdx.x == 0) *out = t;
    }
}

__global__ void k_scale_grid(double *__restrict__ kn, const double *norm)
{
    const int64_t m = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (m < kGrid) kn[m] = kn[m] / *norm;
}

// sm[i] = max(1e-10, sum_{m=0}^{min(i, W)} K[m] dg[i-m]), m ascending per output
__global__ void __launch_bounds__(kConvT) k_conv(const double *__restrict__ K, const unsigned int *lastp,
                                                 const double *__restrict__ dg, double *__restrict__ sm)
{
    __shared__ double kt[kConvT];
    __shared__ double dt[2 * kConvT];
    const int64_t i0 = (int64_t)blockIdx.x * kConvT;
    const int64_t i = i0 + threadIdx.x;
    const int64_t W = (int64_t)*lastp;
    const int64_t top_blk = (i0 + kConvT - 1) < W ? (i0 + kConvT - 1) : W;   // largest m any thread uses
    const int64_t top = i < W ? i : W;
    double s = 0.0;
    for (int64_t m0 = 0; m0 <= top_blk; m0 += kConvT) {
        __syncthreads();
        kt[threadIdx.x] = (m0 + threadIdx.x < kGrid) ? K[m0 + threadIdx.x] : 0.0;
        // dt[q] = dg[i0 - m0 - (kConvT - 1) + q], q in [0, 2 kConvT - 1)
        for (int q = threadIdx.x; q < 2 * kConvT - 1; q += kConvT) {
            const int64_t g = i0 - m0 - (kConvT - 1) + q;
            dt[q] = (g >= 0 && g < kGrid) ? dg[g] : 0.0;
        }
        __syncthreads();
        const int64_t mend = (m0 + kConvT - 1) < top ? (m0 + kConvT - 1) : top;
        for (int64_t m = m0; m <= mend; m++) {
            // dg[i - m] = dt[(i - m) - (i0 - m0 - kConvT + 1)]
            s += kt[m - m0] * dt[(int)(threadIdx.x + kConvT - 1 - (m - m0))];
        }
    }
    sm[i] = s < 1e-10 ? 1e-10 : s;
}

__global__ void k_rho(const double *__restrict__ R, int64_t n, const double *__restrict__ rg,
                      const double *__restrict__ sm, const double *__restrict__ cg, const double *__restrict__ bg,
                      const double *__restrict__ dg, double lmin, double dlog, double *__restrict__ rho)
{
    const double r0 = rg[0], r1 = rg[kGrid - 1];
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x) {
        const double v = R[t];
        if (v <= r0) { rho[t] = sm[0]; continue; }
        if (v >= r1) { rho[t] = sm[kGrid - 1]; continue; }
        // the grid is log-spaced: start from the index log10 gives, then settle it
        int64_t j = (int64_t)((log10(v) - lmin) / dlog);
        j = j < 0 ? 0 : (j > kGrid - 2 ? kGrid - 2 : j);
        while (j > 0 && rg[j] > v) j--;
        while (j < kGrid - 2 && rg[j + 1] <= v) j++;
        const double dx = v - rg[j];
        rho[t] = sm[j] + dx * (bg[j] + dx * (cg[j] + dx * dg[j]));
    }
}

// ---------------------------------------------------------------- records

__global__ void k_pack_sorted(int64_t n, const double *__restrict__ R, const double *__restrict__ V,
                              const double *__restrict__ L, const double *__restrict__ psi,
                              const double *__restrict__ rho, double dM, nsg_rank_sorted *__restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double rr = R[i], v = V[i], l = L[i], p = psi[i];
        nsg_rank_sorted o;
        o.rank = (int32_t)i;
        o.mass = (float)((double)(i + 1) * dM);
        o.r = (float)rr;
        o.vr = (float)v;
        o.psi = (float)p;
        o.E = (float)(p - (l * l / (2.0 * rr * rr)) - 0.5 * v * v);
        o.ell = (float)l;
        o.rho = (float)rho[i];
        out[i] = o;
    }
}

__global__ void k_pack_unsorted(int64_t n, const SnapIn *__restrict__ rec, const double *__restrict__ psi, double dM,
                                nsg_rank_unsorted *__restrict__ out)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const SnapIn s = rec[i];
        const double rr = (double)s.r, v = (double)s.v, l = (double)s.l, p = psi[i];
        nsg_rank_unsorted o;
        o.rank = s.rank;
        o.mass = (float)((double)(s.rank + 1) * dM);
        o.r = s.r;
        o.vr = s.v;
        o.psi = (float)p;
        o.E = (float)(p - (l * l / (2.0 * rr * rr)) - 0.5 * v * v);
        o.ell = s.l;
        out[i] = o;
    }
}

// ---------------------------------------------------------------- orchestration

struct DevBuf {
    std::vector<void *> ptrs;
    cudaStream_t s;
    explicit DevBuf(cudaStream_t st) : s(st) {}
    template <class T> cudaError_t get(T **p, size_t count)
    {
        void *q = nullptr;
        cudaError_t e = cudaMallocAsync(&q, count * sizeof(T) + 16, s);
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = (T *)q;
        return e;
    }
    ~DevBuf()
    {
        for (void *q : ptrs) cudaFreeAsync(q, s);
    }
};

// Smoothed density at the n sorted radii R (device) into rho (device).
static int density(nsg_ctx *c, const double *R, int64_t n, double *rho)
{
    cudaStream_t s = c->stream;
    DevBuf B(s);
    const double dM = c->p.M_total / (double)n;
    const int64_t ntiles = (n + kKeepTile - 1) / kKeepTile;
    long long *cnt = nullptr;
    int32_t *I = nullptr;
    unsigned int *flag = nullptr;
    cudaError_t e = B.get(&cnt, (size_t)ntiles);
    if (e == cudaSuccess) e = B.get(&I, (size_t)n);
    if (e == cudaSuccess) e = B.get(&flag, 4);
    if (e != cudaSuccess) return cuda_err(c, e, "density buffers");
    k_keep_counts<<<(unsigned)ntiles, kKeepThreads, 0, s>>>(R, n, cnt);
    k_scan_ll<<<1, 1024, 0, s>>>(cnt, ntiles);
    k_keep_prefix<<<(unsigned)ntiles, kKeepThreads, 0, s>>>(R, n, cnt, I);
    int32_t F32 = 0;
    e = cudaMemcpyAsync(&F32, I + (n - 1), 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "density subsequence");
    const int64_t F = F32;
    int64_t D = (int64_t)std::ceil((double)n / 100.0);
    if (D > 30000) D = 30000;
    if (D <= 0) D = 1;
    int all = 0;
    double step = 0.0;
    if (F <= D) {
        D = F;
        all = 1;
    } else {
        step = (double)(F - 1) / (double)(D - 1);
    }
    if (D < 3) return set_err(c, NSG_EINVAL, "density needs at least 3 distinct radii after decimation");
    double *Rd, *Md, *cd, *lg, *rg, *mg, *dg, *kn, *sm, *cg, *scratch, *norm;
    unsigned int *last = nullptr;
    const int64_t chunks_max = (kGrid - 2 + kChunk - 1) / kChunk;
    e = B.get(&Rd, (size_t)D);
    if (e == cudaSuccess) e = B.get(&Md, (size_t)D);
    if (e == cudaSuccess) e = B.get(&cd, (size_t)D);
    if (e == cudaSuccess) e = B.get(&lg, kGrid);
    if (e == cudaSuccess) e = B.get(&rg, kGrid);
    if (e == cudaSuccess) e = B.get(&mg, kGrid);
    if (e == cudaSuccess) e = B.get(&dg, kGrid);
    if (e == cudaSuccess) e = B.get(&kn, kGrid);
    if (e == cudaSuccess) e = B.get(&sm, kGrid);
    if (e == cudaSuccess) e = B.get(&cg, kGrid);
    if (e == cudaSuccess) e = B.get(&scratch, (size_t)chunks_max * 2 * (kChunk + 2 * kHalo));
    if (e == cudaSuccess) e = B.get(&norm, 1);
    if (e == cudaSuccess) e = B.get(&last, 1);
    if (e != cudaSuccess) return cuda_err(c, e, "density buffers");
    k_decimate<<<(unsigned)((D + 255) / 256), 256, 0, s>>>(R, I, n, F, D, all, step, dM, Rd, Md);
    double ends[2];
    e = cudaMemcpyAsync(&ends[0], Rd, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&ends[1], Rd + (D - 1), 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "density decimation");
    // the reference's validation (:7363-7374)
    if (!(ends[0] > 0.0) || !(ends[1] > ends[0]) || !std::isfinite(ends[1]))
        return set_err(c, NSG_EINVAL, "density needs a positive smallest radius and a finite range");
    const double min_r = ends[0], max_r = ends[1] * 1.04;
    const double lmin = std::log10(min_r), lmax = std::log10(max_r);
    const double dlog = (lmax - lmin) / (double)(kGrid - 1);
    const unsigned gb = (unsigned)((kGrid + 255) / 256);
    auto mono = [&](double *x, int64_t m) -> cudaError_t {
        unsigned int h = 0;
        cudaError_t e2 = cudaMemsetAsync(flag, 0, 4, s);
        k_mono_check<<<gb, 256, 0, s>>>(x, m, flag);
        if (e2 == cudaSuccess) e2 = cudaMemcpyAsync(&h, flag, 4, cudaMemcpyDeviceToHost, s);
        if (e2 == cudaSuccess) e2 = cudaStreamSynchronize(s);
        if (e2 == cudaSuccess && h) k_mono_fix<<<1, 1, 0, s>>>(x, m);
        return e2;
    };
    k_grid<<<gb, 256, 0, s>>>(lmin, dlog, lg, rg);
    e = mono(rg, kGrid);
    if (e == cudaSuccess) e = mono(Rd, D);
    if (e != cudaSuccess) return cuda_err(c, e, "density grid");
    k_cspline_chunks<<<(unsigned)(((D - 2 + kChunk - 1) / kChunk + 127) / 128), 128, 0, s>>>(Rd, Md, D, cd, scratch);
    k_mass_grid<<<gb, 256, 0, s>>>(rg, Rd, Md, cd, D, mg);
    unsigned int hf = 0;
    e = cudaMemsetAsync(flag, 0, 4, s);
    k_dens_grid<<<gb, 256, 0, s>>>(rg, mg, dg, flag);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hf, flag, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "density gradient");
    if (hf) k_dens_grid_seq<<<1, 1, 0, s>>>(rg, mg, dg);
    k_dens_ends<<<1, 1, 0, s>>>(dg);
    // smoothing (:7539-7570): sigma in log10 r, taps at multiples of the grid step
    const double sigma = 0.08 * std::pow((double)n / 10000.0, -0.40);
    const double l1 = lmin + 1.0 * dlog;
    const double tap = l1 - lmin;
    const double pref = 1.0 / (sigma * std::sqrt(2.0 * M_PI));
    e = cudaMemsetAsync(last, 0, 4, s);
    if (e != cudaSuccess) return cuda_err(c, e, "density smoothing");
    k_gauss<<<gb, 256, 0, s>>>(tap, sigma, pref, kn, last);
    k_sum_grid<<<1, 1024, 0, s>>>(kn, norm);
    k_scale_grid<<<gb, 256, 0, s>>>(kn, norm);
    k_conv<<<(unsigned)(kGrid / kConvT), kConvT, 0, s>>>(kn, last, dg, sm);
    k_cspline_chunks<<<(unsigned)((chunks_max + 127) / 128), 128, 0, s>>>(rg, sm, kGrid, cg, scratch);
    // the interval coefficients reuse buffers the smoothing no longer needs
    double *bgc = kn, *dgc = mg;
    k_cs_coef<<<gb, 256, 0, s>>>(rg, sm, cg, kGrid, bgc, dgc);
    k_rho<<<grid_for(c, n, 256), 256, 0, s>>>(R, n, rg, sm, cg, bgc, dgc, lmin, dlog, rho);
    c->launches += 21;
    e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "density");
}

}  // namespace nsg

using namespace nsg;

extern "C" int nsg_post_snapshot(nsg_ctx *c, const void *records, int64_t n, nsg_rank_sorted *sorted_out,
                                 nsg_rank_unsorted *unsorted_out, double *psi0)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (!records || n <= 0) return set_err(c, NSG_EINVAL, "records missing");
    if (int rc = begin_upload(c, n)) return rc;
    cudaStream_t s = c->stream;
    DevBuf B(s);
    SnapIn *rec = nullptr;
    double *knots = nullptr, *psiK = nullptr, *Esc = nullptr, *psiS = nullptr, *psiU = nullptr, *rho = nullptr;
    double *tile = nullptr, *total = nullptr;
    cudaError_t e = B.get(&rec, (size_t)n);
    if (e == cudaSuccess) e = B.get(&knots, (size_t)n + 1);
    if (e == cudaSuccess) e = B.get(&psiK, (size_t)n + 1);
    if (e == cudaSuccess) e = B.get(&Esc, (size_t)n);
    if (e == cudaSuccess) e = B.get(&psiS, (size_t)n);
    if (e == cudaSuccess) e = B.get(&psiU, (size_t)n);
    if (e == cudaSuccess) e = B.get(&rho, (size_t)n);
    if (e == cudaSuccess) e = B.get(&tile, (size_t)post_tiles(n));
    if (e == cudaSuccess) e = B.get(&total, 1);
    if (e != cudaSuccess) return cuda_err(c, e, "post-processing buffers");
    {
        ProfScope ps(c, "post_h2d", (double)n * sizeof(SnapIn));
        e = cudaMemcpyAsync(rec, records, (size_t)n * sizeof(SnapIn), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) return cuda_err(c, e, "post-processing upload");
    }
    {
        ProfScope ps(c, "post_unpack", (double)n * (16 + 28));
        k_snap_to_state<<<grid_for(c, n, 256), 256, 0, s>>>(rec, n, c->r[0], c->vr[0], c->ell[0], c->id[0]);
        c->launches += 1;
    }
    if (int rc = sort_state(c)) return rc;
    const int k = c->cur;
    const double *R = c->r[k], *V = c->vr[k], *L = c->ell[k];
    // the knot adjustment (one warp, the longest stage) runs on the side stream
    // beside the density and the potential
    e = cudaEventRecord(c->ev_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
    if (e != cudaSuccess) return cuda_err(c, e, "post-processing fork");
    {
        ProfScope ps(c, "post_knots", (double)n * 16, c->side);
        k_psi_knots<<<1, 32, 0, c->side>>>(R, n, knots);
        c->launches += 1;
    }
    e = cudaEventRecord(c->ev_join, c->side);
    if (e != cudaSuccess) return cuda_err(c, e, "post-processing join");
    // on every return from here the buffers are freed on the main stream (B's
    // destructor) only after the side stream's warp is done with them
    struct JoinGuard {
        cudaStream_t st;
        cudaEvent_t ev;
        ~JoinGuard() { cudaStreamWaitEvent(st, ev, 0); }
    } join_guard{s, c->ev_join};
    {
        ProfScope ps(c, "post_density", (double)n * 24);
        if (int rc = density(c, R, n, rho)) return rc;
    }
    const double dM = c->p.M_total / (double)n;
    {
        ProfScope ps(c, "post_psi", (double)n * 40);
        if (int rc = post_psi_sorted(c, R, V, L, n, psiK + 1, Esc, tile, total)) return rc;
        k_set_psi0<<<1, 1, 0, s>>>(psiK, total, c->p.G, dM);
        c->launches += 1;
    }
    e = cudaStreamWaitEvent(s, c->ev_join, 0);
    if (e != cudaSuccess) return cuda_err(c, e, "post-processing join");
    {
        ProfScope ps(c, "post_interp", (double)n * 48);
        k_psi_interp<<<grid_for(c, n, 256), 256, 0, s>>>(knots, psiK, n + 1, R, nullptr, n, psiS);
        k_psi_interp<<<grid_for(c, n, 256), 256, 0, s>>>(knots, psiK, n + 1, nullptr, rec, n, psiU);
        c->launches += 2;
    }
    nsg_rank_sorted *ds = nullptr;
    nsg_rank_unsorted *du = nullptr;
    if (sorted_out) e = B.get(&ds, (size_t)n);
    if (e == cudaSuccess && unsorted_out) e = B.get(&du, (size_t)n);
    if (e != cudaSuccess) return cuda_err(c, e, "post-processing buffers");
    {
        ProfScope ps(c, "post_pack", (double)n * (sorted_out ? 72 : 0) + (double)n * (unsorted_out ? 52 : 0));
        if (ds) k_pack_sorted<<<grid_for(c, n, 256), 256, 0, s>>>(n, R, V, L, psiS, rho, dM, ds);
        if (du) k_pack_unsorted<<<grid_for(c, n, 256), 256, 0, s>>>(n, rec, psiU, dM, du);
        c->launches += (ds ? 1 : 0) + (du ? 1 : 0);
    }
    {
        ProfScope ps(c, "post_d2h", (double)n * ((ds ? 32 : 0) + (du ? 28 : 0)));
        if (ds) e = cudaMemcpyAsync(sorted_out, ds, (size_t)n * sizeof(nsg_rank_sorted), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess && du)
            e = cudaMemcpyAsync(unsorted_out, du, (size_t)n * sizeof(nsg_rank_unsorted), cudaMemcpyDeviceToHost, s);
    }
    double h0 = 0.0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h0, psiK, 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "post-processing");
    if (psi0) *psi0 = h0;
    if (c->profiling) prof_flush(c);
    return NSG_OK;
}
