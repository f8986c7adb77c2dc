// nsg_bucket.cu -- near-sorted bucket sort: the fast path of the radial sort.
//
// Between steps every particle moves a small distance in r, so the state arrives
// almost in (r, id) order.  The sort exploits that instead of re-sorting all 64
// key bits (nsphere.c relies on the same property: quadsort is adaptive to
// ordered runs, README "nearly N log N or even linear"):
//
//   splitters  S[b] = key(r) at sorted position b*B of the previous sort (written
//              by the pass that consumed that sort), so S is non-decreasing;
//   scatter    each particle finds its bucket b (S[b] <= key < S[b+1]) by a short
//              search from its home bucket i/B, and appends (key, id, index) to a
//              fixed-capacity bucket slot array;
//   scan       exclusive scan of the bucket counts; a count above the capacity
//              sets the fallback flag, and the general radix sort runs instead;
//   sort       one block per bucket sorts its entries in registers/shared memory
//              by a stable LSD radix over only the key bits that differ inside
//              the bucket (typically 40 of 64), then by id where keys tie, and
//              writes the source index of each sorted position.
// The concatenation of sorted buckets is the (r, id) order: buckets partition the
// key range in splitter order and equal keys share a bucket.
#include "nsg_internal.cuh"

namespace nsg {

constexpr int kBucketThreads = 1024;
constexpr int kBucketItems = 6;
constexpr int kBucketWarps = kBucketThreads / 32;


// Largest b in [lo, hi) with S(b) <= key (S(lo) is the smallest key of the halo),
// searched from home; S(b) gives splitter b.
template <typename SplitFn>
__device__ __forceinline__ int find_bucket_f(SplitFn S, int lo0, int hi0, uint64_t key, int home)
{
    int b = home;
    if (S(b) <= key) {
        int steps = 0;
        while (b + 1 < hi0 && S(b + 1) <= key && steps < 8) { b++; steps++; }
        if (b + 1 < hi0 && S(b + 1) <= key) {      // far move: binary search in (b, hi0)
            int lo = b + 1, hi = hi0 - 1;          // S(lo) <= key
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (S(mid) <= key) lo = mid; else hi = mid - 1;
            }
            b = lo;
        }
    } else {
        int steps = 0;
        while (b > lo0 && S(b) > key && steps < 8) { b--; steps++; }
        if (S(b) > key) {                          // binary search in [lo0, b)
            int lo = lo0, hi = b - 1;              // S(lo0) <= key always
            while (lo < hi) {
                int mid = (lo + hi + 1) >> 1;
                if (S(mid) <= key) lo = mid; else hi = mid - 1;
            }
            b = lo;
        }
    }
    return b;
}

__device__ __forceinline__ int find_bucket(const uint64_t *__restrict__ S, int lo0, int hi0, uint64_t key, int home)
{
    return find_bucket_f([S](int b) { return S[b]; }, lo0, hi0, key, home);
}

__global__ void __launch_bounds__(256)
k_bucket_scatter(const double *__restrict__ r, const int32_t *__restrict__ id, int64_t n,
                 const uint64_t *__restrict__ S, Seg sg, int B, int cap,
                 unsigned int *__restrict__ cnt, uint64_t *__restrict__ bkey,
                 uint64_t *__restrict__ bpay, DevCounters *ctr)
{
    bool nan_seen = false;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        double rp = r[p];
        nan_seen |= (rp != rp);
        uint64_t key = radius_key(rp);
        // a particle stays in its halo: search that halo's buckets only
        const Local L = local_of(sg, p, n);
        const int lo = sg.bbase[L.h], hi = sg.bbase[L.h + 1];
        int home = lo + (int)(L.i / B);
        if (home >= hi) home = hi - 1;
        int b = find_bucket(S, lo, hi, key, home);
        unsigned active = __activemask();
        unsigned peers = __match_any_sync(active, b);
        int leader = __ffs(peers) - 1;
        unsigned base = 0;
        if ((int)(threadIdx.x & 31) == leader) base = atomicAdd(&cnt[b], (unsigned)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        unsigned slot = base + __popc(peers & lanemask_lt());
        if (slot < (unsigned)cap) {
            int64_t at = (int64_t)b * cap + slot;
            bkey[at] = key;
            bpay[at] = ((uint64_t)(uint32_t)id[p] << 32) | (uint64_t)(uint32_t)p;
        }
    }
    if (nan_seen) atomicOr(&ctr->status, NSG_ST_NAN);
}

// Index scatter of the fused path, 8 particles per thread: a block takes 2048
// consecutive positions and loads all their radii first (coalesced), and, beside
// them, the splitters of the home buckets those positions map to (one halo:
// position >> bshift; at most six for bucket targets of 512 and up) into shared
// memory.  Each particle then tests its home bucket with both bounding splitters --
// the common case, a particle that did not cross a splitter -- and walks or searches
// only when it did.  The appends: a warp whose particles all fall in one bucket takes
// its slots with one atomic, in position order.  Counts go to the low word of the
// bucket's look-back word (cnt[2 b]); a particle past its bucket's capacity sets *over
// and the fallback status (the consumer then hands the sort to the radix path).
// COLLECT: the same pass lists the Levi-Civita candidates (radius key below lc.kthr)
// for k_lc_early_rank, as k_lc_early_collect does.
constexpr int kScatterItems = 8;
constexpr int kScatterHomes = 8;                       // cached splitters [hb0, hb0 + 8)

struct LcCollect {
    uint64_t kthr;
    uint64_t *ckey;
    int32_t *cid;
    uint32_t *csrc;
    const int32_t *id_src;
};

template <bool COLLECT>
__global__ void __launch_bounds__(256, 6)
k_bucket_scatter_idx(const double *__restrict__ r, int64_t n, const uint64_t *__restrict__ S, Seg sg, int bshift,
                     int cap, unsigned int *__restrict__ cnt, unsigned int *__restrict__ over,
                     uint32_t *__restrict__ bidx, DevCounters *ctr, LcCollect lc)
{
    __shared__ uint64_t sS[kScatterHomes];
    const int64_t p0 = (int64_t)blockIdx.x * (256 * kScatterItems);
    const bool one = sg.nseg <= 1;
    const int hb0 = (int)(p0 >> bshift);
    double rv[kScatterItems];
#pragma unroll
    for (int j = 0; j < kScatterItems; j++) {
        const int64_t p = p0 + j * 256 + threadIdx.x;
        rv[j] = p < n ? r[p] : 0.0;
    }
    if (one && threadIdx.x < kScatterHomes) {
        const int h = hb0 + (int)threadIdx.x;
        sS[threadIdx.x] = h < sg.bbase[1] ? S[h] : ~0ull;   // entries past the last bucket are never read
    }
    __syncthreads();
    bool nan_seen = false, overflow = false;
    const int lane = threadIdx.x & 31;
    const int64_t wp0 = p0 + (threadIdx.x & ~31u);     // position of lane 0 at j = 0
#pragma unroll
    for (int j = 0; j < kScatterItems; j++) {
        if (wp0 + j * 256 >= n) break;                 // uniform: the rest of the warp's items are past the end
        const int64_t p = p0 + j * 256 + threadIdx.x;
        const bool valid = p < n;                      // a prefix of the warp's lanes, lane 0 among them
        int b = -1;
        uint64_t key = ~0ull;
        if (valid) {
            key = radius_key(rv[j]);
            nan_seen |= (key == ~0ull);          // NaN, tested on the integer pipe
            const Local L = local_of(sg, p, n);
            const int lo = sg.bbase[L.h], hi = sg.bbase[L.h + 1];
            int home = lo + (int)(L.i >> bshift);
            if (home >= hi) home = hi - 1;
            const int q = home - hb0;
            uint64_t s0, s1;
            if (one && q >= 0 && q + 1 < kScatterHomes) {
                s0 = sS[q];
                s1 = home + 1 < hi ? sS[q + 1] : ~0ull;
            } else {
                s0 = S[home];
                s1 = home + 1 < hi ? S[home + 1] : ~0ull;
            }
            if (s0 <= key && (key < s1 || home + 1 >= hi)) b = home;
            else b = find_bucket(S, lo, hi, key, home);
        }
        if (COLLECT) {
            const bool cand = valid && key < lc.kthr;
            if (__any_sync(0xffffffffu, cand)) {
                const int slot = warp_append(cand, &ctr->lc_cand);
                if (cand && slot < kLcEarlyCap) {
                    lc.ckey[slot] = key;
                    lc.cid[slot] = lc.id_src[p];
                    lc.csrc[slot] = (uint32_t)p;
                }
            }
        }
        // slots: a warp whose particles all fall in one bucket takes them with one
        // atomic; otherwise the leader of each group of lanes with one bucket does
        const int b0 = __shfl_sync(0xffffffffu, b, 0);
        unsigned peers;
        int leader = 0;
        if (__all_sync(0xffffffffu, !valid || b == b0)) {
            peers = __ballot_sync(0xffffffffu, valid);
        } else {
            peers = __match_any_sync(0xffffffffu, b);
            leader = __ffs(peers) - 1;
        }
        unsigned base = 0;
        if (lane == leader && valid) base = atomicAdd(&cnt[2 * b], (unsigned)__popc(peers));
        base = __shfl_sync(0xffffffffu, base, leader);
        const unsigned slot = base + __popc(peers & lanemask_lt());
        const bool fits = slot < (unsigned)cap;
        if (valid && fits) bidx[(int64_t)b * cap + slot] = (uint32_t)p;
        overflow |= valid && !fits;
    }
    if (__any_sync(0xffffffffu, overflow) && lane == 0) {
        *over = 1u;
        atomicOr(&ctr->status, NSG_ST_SORT_FALLBACK);
    }
    if (nan_seen) atomicOr(&ctr->status, NSG_ST_NAN);
}

// Exclusive scan of the bucket counts (one block); flags overflow.
__global__ void __launch_bounds__(1024)
k_bucket_scan(const unsigned int *__restrict__ cnt, int nb, int cap, unsigned int *__restrict__ off,
              DevCounters *ctr)
{
    __shared__ unsigned int wt[32];
    __shared__ unsigned int carry_s;
    __shared__ int over_s;
    if (threadIdx.x == 0) { carry_s = 0; over_s = 0; }
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int t0 = 0; t0 < nb; t0 += 1024) {
        int t = t0 + threadIdx.x;
        unsigned v = t < nb ? cnt[t] : 0u;
        if (v > (unsigned)cap) over_s = 1;
        unsigned x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) wt[w] = x;
        __syncthreads();
        if (w == 0) {
            unsigned s = wt[lane], tot = s;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                unsigned y = __shfl_up_sync(0xffffffffu, tot, o);
                if (lane >= o) tot += y;
            }
            wt[lane] = tot - s;
        }
        __syncthreads();
        if (t < nb) off[t] = carry_s + wt[w] + x - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry_s += wt[w] + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        ctr->need_fallback = over_s ? 1u : 0u;
        if (over_s) atomicOr(&ctr->status, NSG_ST_SORT_FALLBACK);
    }
}

// One stable LSD pass on 8 bits chosen by `digit_of`, over the block's items held
// in registers.  Warp w owns positions [w*S, (w+1)*S) with S = J*32: item j < J of
// lane l is position w*S + j*32 + l, so walking j and then lanes visits positions
// in order and the match.any ranks are stable.  J = ceil(count / 1024) adapts the
// work to the bucket's fill; items are exchanged through shared memory.
template <typename DigitFn>
__device__ __forceinline__ void block_radix_pass(uint64_t (&k)[kBucketItems], uint64_t (&v)[kBucketItems],
                                                 int J, DigitFn digit_of, uint32_t (*whist)[256],
                                                 uint32_t *dtot, uint64_t *xk)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int S = J * 32;
    const unsigned lt = lanemask_lt();
    for (int d = threadIdx.x; d < kBucketWarps * 256; d += blockDim.x) (&whist[0][0])[d] = 0;
    __syncthreads();
    uint32_t rd[kBucketItems];   // (rank within warp and digit) << 8 | digit
#pragma unroll
    for (int j = 0; j < kBucketItems; j++) {
        if (j < J) {
            unsigned d = digit_of(k[j], v[j]);
            unsigned peers = __match_any_sync(0xffffffffu, d);
            uint32_t c = whist[w][d];
            rd[j] = ((c + __popc(peers & lt)) << 8) | d;
            __syncwarp();
            if (lane == __ffs(peers) - 1) whist[w][d] = c + __popc(peers);
            __syncwarp();
        }
    }
    __syncthreads();
    // digit-major exclusive offsets: per digit over warps, then over digits
    if (threadIdx.x < 256) {
        const int d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kBucketWarps; ww++) {
            uint32_t t = whist[ww][d];
            whist[ww][d] = run;
            run += t;
        }
        dtot[d] = run;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        // scan of 256 digit totals by one warp: 8 per lane
        uint32_t loc[8], s = 0;
#pragma unroll
        for (int q = 0; q < 8; q++) { loc[q] = dtot[lane * 8 + q]; s += loc[q]; }
        uint32_t x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        uint32_t run = x - s;
#pragma unroll
        for (int q = 0; q < 8; q++) { dtot[lane * 8 + q] = run; run += loc[q]; }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBucketItems; j++) {
        if (j < J) {
            const uint32_t d = rd[j] & 255u;
            xk[dtot[d] + whist[w][d] + (rd[j] >> 8)] = k[j];
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBucketItems; j++)
        if (j < J) k[j] = xk[w * S + j * 32 + lane];
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBucketItems; j++) {
        if (j < J) {
            const uint32_t d = rd[j] & 255u;
            xk[dtot[d] + whist[w][d] + (rd[j] >> 8)] = v[j];
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kBucketItems; j++)
        if (j < J) v[j] = xk[w * S + j * 32 + lane];
    __syncthreads();
}

__device__ __forceinline__ uint64_t block_reduce_u64(uint64_t x, bool is_min, uint64_t *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        uint64_t y = __shfl_xor_sync(0xffffffffu, x, o);
        x = is_min ? (y < x ? y : x) : (y > x ? y : x);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[w] = x;
    __syncthreads();
    x = red[0];
    for (int i = 1; i < kBucketWarps; i++) {
        uint64_t y = red[i];
        x = is_min ? (y < x ? y : x) : (y > x ? y : x);
    }
    return x;
}

__global__ void __launch_bounds__(kBucketThreads)
k_bucket_sort(const unsigned int *__restrict__ cnt, const unsigned int *__restrict__ off, int cap,
              const uint64_t *__restrict__ bkey, const uint64_t *__restrict__ bpay,
              uint32_t *__restrict__ perm, const DevCounters *__restrict__ ctr)
{
    if (ctr->need_fallback) return;
    extern __shared__ __align__(16) unsigned char smem[];
    uint64_t *xk = reinterpret_cast<uint64_t *>(smem);                      // cap * 8
    uint32_t(*whist)[256] = reinterpret_cast<uint32_t(*)[256]>(xk + cap);   // warps * 256 * 4
    uint32_t *dtot = &whist[kBucketWarps - 1][0] + 256;                      // 256 * 4
    __shared__ uint64_t red[kBucketWarps];

    const int b = blockIdx.x;
    const uint32_t m = cnt[b];
    if (m == 0) return;
    const uint32_t base = off[b];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int J = (int)((m + kBucketThreads - 1) / kBucketThreads);   // 1 .. kBucketItems
    const int S = J * 32;
    const int64_t src0 = (int64_t)b * cap;
    uint64_t k[kBucketItems], v[kBucketItems];
    uint64_t kmin = ~0ull, kmax = 0ull;
#pragma unroll
    for (int j = 0; j < kBucketItems; j++) {
        const uint32_t pos = w * S + j * 32 + lane;
        const bool ok = (j < J) && pos < m;
        k[j] = ok ? bkey[src0 + pos] : ~0ull;
        v[j] = ok ? bpay[src0 + pos] : ~0ull;
        if (ok) { kmin = k[j] < kmin ? k[j] : kmin; kmax = k[j] > kmax ? k[j] : kmax; }
    }
    kmin = block_reduce_u64(kmin, true, red);
    kmax = block_reduce_u64(kmax, false, red);
    const uint64_t diff = kmin ^ kmax;
    const int kbits = diff ? 64 - __clzll((long long)diff) : 0;
    if (kbits > 16) {
        // Fast form: two passes on a 16-bit quantised key q = (key - kmin) >> qs (monotone
        // in the key), then each run of equal q -- a few elements at most for keys spread
        // over 2^40 values -- is ordered by (key, id) by counting ranks.  A run longer than
        // 32 sends the block to the full form below (any start order is fine for it).
        // padding items (key ~0, positions >= m) clamp to the top value and, the passes
        // being stable, stay behind every real item
        const int qb = 64 - __clzll((long long)(kmax - kmin));
        const int qs = qb > 16 ? qb - 16 : 0;
        const uint64_t k0 = kmin;
        for (int shift = 0; shift < 16; shift += 8)
            block_radix_pass(k, v, J, [shift, qs, k0](uint64_t kk, uint64_t) {
                const uint64_t q = (kk - k0) >> qs;
                return (unsigned)((q < 0xffffull ? q : 0xffffull) >> shift) & 255u; }, whist, dtot, xk);
        uint32_t fin[kBucketItems];
        int too_long = 0;
#pragma unroll
        for (int j = 0; j < kBucketItems; j++)
            if (j < J) xk[w * S + j * 32 + lane] = k[j];
        __syncthreads();
        uint32_t rs[kBucketItems], eqm[kBucketItems];   // run start | length << 16, equal-key mask
#pragma unroll
        for (int j = 0; j < kBucketItems; j++) {
            const uint32_t pos = w * S + j * 32 + lane;
            fin[j] = pos;
            rs[j] = pos;
            eqm[j] = 0;
            if (j < J && pos < m) {
                const uint64_t q = (k[j] - k0) >> qs;
                uint32_t lo = pos, hi = pos + 1;
                while (lo > 0 && pos - lo < 33 && ((xk[lo - 1] - k0) >> qs) == q) lo--;
                while (hi < m && hi - pos < 33 && ((xk[hi] - k0) >> qs) == q) hi++;
                const uint32_t len = hi - lo;
                if (len > 32) too_long = 1;
                else if (len > 1) {
                    uint32_t less = 0, eq = 0;
                    for (uint32_t t = 0; t < len; t++) {
                        const uint64_t kq = xk[lo + t];
                        less += kq < k[j];
                        if (kq == k[j] && lo + t != pos) eq |= 1u << t;
                    }
                    fin[j] = lo + less;
                    rs[j] = lo | (len << 16);
                    eqm[j] = eq;
                }
            }
        }
        too_long = __syncthreads_or(too_long);
        if (!too_long) {
            // equal keys inside a run: by id (ids are distinct)
#pragma unroll
            for (int j = 0; j < kBucketItems; j++)
                if (j < J) xk[w * S + j * 32 + lane] = v[j];
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kBucketItems; j++) {
                if (j < J && eqm[j]) {
                    const uint32_t lo = rs[j] & 0xffffu, id = (uint32_t)(v[j] >> 32);
                    uint32_t e = eqm[j], add = 0;
                    while (e) {
                        const int t = __ffs(e) - 1;
                        e &= e - 1;
                        add += (uint32_t)(xk[lo + t] >> 32) < id;
                    }
                    fin[j] += add;
                }
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kBucketItems; j++) {
                const uint32_t pos = w * S + j * 32 + lane;
                if (j < J && pos < m) xk[fin[j]] = v[j];
            }
            __syncthreads();
#pragma unroll
            for (int j = 0; j < kBucketItems; j++) {
                const uint32_t pos = w * S + j * 32 + lane;
                if (j < J && pos < m) perm[base + pos] = (uint32_t)(xk[pos] & 0xffffffffu);
            }
            return;
        }
        __syncthreads();
    }
    for (int shift = 0; shift < kbits; shift += 8)
        block_radix_pass(k, v, J, [shift](uint64_t kk, uint64_t) { return (unsigned)(kk >> shift) & 255u; },
                         whist, dtot, xk);
    // ties on the key (equal radii) are ordered by id: re-sort by id, then by key
    int tie = 0;
    {
#pragma unroll
        for (int j = 0; j < kBucketItems; j++)
            if (j < J) xk[w * S + j * 32 + lane] = k[j];
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kBucketItems; j++) {
            const uint32_t pos = w * S + j * 32 + lane;
            if (j < J && pos + 1 < m && xk[pos] == xk[pos + 1]) tie = 1;
        }
        tie = __syncthreads_or(tie);
    }
    if (tie) {
        uint64_t imin = ~0ull, imax = 0ull;
#pragma unroll
        for (int j = 0; j < kBucketItems; j++) {
            const uint32_t pos = w * S + j * 32 + lane;
            if (j < J && pos < m) {
                const uint64_t x = v[j] >> 32;
                imin = x < imin ? x : imin;
                imax = x > imax ? x : imax;
            }
        }
        imin = block_reduce_u64(imin, true, red);
        imax = block_reduce_u64(imax, false, red);
        const uint64_t idiff = imin ^ imax;
        const int ibits = idiff ? 64 - __clzll((long long)idiff) : 0;
        for (int shift = 0; shift < ibits; shift += 8)
            block_radix_pass(k, v, J, [shift](uint64_t, uint64_t vv) { return (unsigned)((vv >> 32) >> shift) & 255u; },
                             whist, dtot, xk);
        for (int shift = 0; shift < kbits; shift += 8)
            block_radix_pass(k, v, J, [shift](uint64_t kk, uint64_t) { return (unsigned)(kk >> shift) & 255u; },
                             whist, dtot, xk);
    }
#pragma unroll
    for (int j = 0; j < kBucketItems; j++) {
        const uint32_t pos = w * S + j * 32 + lane;
        if (j < J && pos < m) perm[base + pos] = (uint32_t)(v[j] & 0xffffffffu);
    }
}

size_t bucket_smem_bytes(int cap)
{
    return (size_t)cap * 8 + (size_t)kBucketWarps * 256 * 4 + 256 * 4;
}

// Slot capacity of a bucket on the two-kernel path: three times the bucket target,
// rounded up to whole 1024-thread rows of k_bucket_sort (which writes its padding
// items too), at most kBucketCap.
int bucket_cap(const nsg_ctx *c)
{
    const int want = ((3 << c->tune.bshift) + 1023) & ~1023;
    return want < kBucketCap ? want : kBucketCap;
}

// Fast path of the sort.  Returns NSG_OK having launched the bucket kernels; the
// radix kernels that follow run only if the scan flagged an overflow.
int bucket_sort_perm(nsg_ctx *c)
{
    const int64_t n = c->n;
    const int src = c->cur;
    const int B = 1 << c->tune.bshift, cap = bucket_cap(c);
    const int nb = (int)c->nb_total;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemsetAsync(c->bcnt, 0, (size_t)nb * 4, s);
    if (e != cudaSuccess) return cuda_err(c, e, "bucket count reset");
    {
        ProfScope ps(c, "bucket_scatter", (double)n * (8 + 4 + 16));
        k_bucket_scatter<<<grid_for(c, n, 256, 8), 256, 0, s>>>(c->r[src], c->id[src], n, c->split, seg_table(c),
                                                                 B, cap, c->bcnt, c->bkey, c->bpay, c->ctr);
        k_bucket_scan<<<1, 1024, 0, s>>>(c->bcnt, nb, cap, c->boff, c->ctr);
    }
    {
        ProfScope ps(c, "bucket_sort", (double)n * (16 + 4));
        k_bucket_sort<<<nb, kBucketThreads, bucket_smem_bytes(cap), s>>>(c->bcnt, c->boff, cap, c->bkey,
                                                                        c->bpay, c->vals[0], c->ctr);
    }
    c->launches += 3;
    e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "bucket sort kernels");
}

// Entries a fused block sorts: twice the bucket target, 0 when the bucket target is
// above what one block holds (the fused kernels are then not used).
int fused_cap(const nsg_ctx *c)
{
    // blocks of 128, 256 or 512 threads holding 8 entries each
    return (c->tune.bshift >= 9 && c->tune.bshift <= 11) ? (2 << c->tune.bshift) : 0;
}

bool use_fused(const nsg_ctx *c)
{
    return c->split_valid && c->p.sort_mode == 0 && fused_cap(c) > 0;
}

// Scatter of the fused path: after this, bucket b's particle indices are in
// c->bidx[b * cap ..] and its count in the low word of its look-back word
// (FusedSort); an overfull bucket sets the overflow word, and the fused kernel then
// sets need_fallback and returns at once (the radix sort with the two-kernel
// consumers runs instead).  The bucket starts are found inside the fused kernel.
int bucket_fused_prepare(nsg_ctx *c, cudaStream_t s, uint64_t lc_thr)
{
    const int64_t n = c->n;
    const int src = c->cur;
    const int cap = fused_cap(c);
    const int nb = (int)c->nb_total;
    // look-back words [nb] and the overflow word (+ pad)
    cudaError_t e = cudaMemsetAsync(c->bcnt, 0, (size_t)nb * 8 + 8, s);
    if (e != cudaSuccess) return cuda_err(c, e, "bucket count reset");
    {
        ProfScope ps(c, "bucket_scatter", (double)n * (8 + 4), s);
        const int64_t blocks = (n + 256 * kScatterItems - 1) / (256 * kScatterItems);
        LcCollect lc{lc_thr, nullptr, nullptr, nullptr, c->id[src]};
        if (lc_thr) {   // the early Levi-Civita list's candidate arrays (keys, ids, sources)
            lc.ckey = reinterpret_cast<uint64_t *>(c->lc_early);
            lc.cid = reinterpret_cast<int32_t *>(c->lc_early + (size_t)kLcEarlyCap * 8);
            lc.csrc = reinterpret_cast<uint32_t *>(c->lc_early + (size_t)kLcEarlyCap * 12);
        }
        if (lc_thr)
            k_bucket_scatter_idx<true><<<(unsigned)blocks, 256, 0, s>>>(c->r[src], n, c->split, seg_table(c),
                                                                         c->tune.bshift, cap, c->bcnt, c->bcnt + 2 * nb,
                                                                         c->bidx, c->ctr, lc);
        else
            k_bucket_scatter_idx<false><<<(unsigned)blocks, 256, 0, s>>>(c->r[src], n, c->split, seg_table(c),
                                                                          c->tune.bshift, cap, c->bcnt, c->bcnt + 2 * nb,
                                                                          c->bidx, c->ctr, lc);
    }
    c->launches += 1;
    e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "bucket scatter kernels");
}

int bucket_setup(nsg_ctx *c)
{
    cudaError_t e = cudaFuncSetAttribute(k_bucket_sort, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)bucket_smem_bytes(kBucketCap));
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "bucket sort attribute");
}

}  // namespace nsg
