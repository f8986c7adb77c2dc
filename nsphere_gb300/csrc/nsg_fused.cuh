// nsg_fused.cuh -- the near-sorted sort done inside the kernel that consumes it.
//
// The scatter pass (k_bucket_scatter_idx, nsg_bucket.cu) leaves, for every bucket b
// of the previous sort's splitters, the source indices of the particles whose key
// falls in [S[b], S[b+1]) in bidx[b * cap ..].  One block per bucket then
//   1. loads the indices, and through them r and id (coalesced in near-sorted order);
//   2. counting-sorts its entries on a quantised key q = (key - kmin) >> qs,
//      monotone in the key, with as many bins as the block holds entries, into
//      shared memory;
//   3. orders each bin holding more than one entry by (key, id) by counting ranks
//      (bins hold ~1 entry for keys spread over the bucket's range); a bin above
//      kFixupMax entries -- many equal radii, or keys bunched by an outlier -- sends
//      the block to a bitonic sort of its entries by (key, id) in shared memory;
//   4. hands sorted position j of the bucket (global position off[b] + j, off[b] found
//      by a look-back over the bucket counts, lookback_partial) with its
//      r, id and source index to the kernel's own per-particle work (rank force,
//      kick, adaptive level 0), which gathers the rest of the particle by the index.
// The concatenation of the sorted buckets is the (r, id) order of the whole halo:
// buckets partition the key range in splitter order and equal keys share a bucket.
// Nothing but the per-particle outputs goes back to memory (no permutation array).
#pragma once
#include "nsg_internal.cuh"

namespace nsg {

constexpr int kFusedItems = 8;                    // entries per thread; a block of T threads holds
                                                  // cap = 8 T entries and quantises keys to cap bins
constexpr int kFixupMax = 32;                     // largest bin ordered by counting ranks

// Dynamic shared memory of a block that sorts up to `cap` entries.
// Layout: keys [cap] | entries [cap] | bin offsets [cap + 1] (+1 pad) | 48 reduction
// words (per warp: minimum, maximum, look-back partials).
__host__ __device__ constexpr size_t fused_smem_bytes(int cap)
{
    return (size_t)cap * 16 + (size_t)(cap + 2) * 4 + 48 * 8;
}

__host__ __device__ constexpr int fused_log2(int x) { return x <= 1 ? 0 : 1 + fused_log2(x >> 1); }

// Per bucket b, look[b] holds its entry count in the low word (added up by the
// scatter) and, once block b has found where the bucket starts, 1 + its inclusive
// prefix (the sorted position one past its last entry) in the high word; 0 there
// means not yet published.  *over is set by the scatter when a bucket overflowed.
struct FusedSort {
    const uint32_t *bidx;        // [nb * cap] source indices per bucket
    unsigned long long *look;    // [nb] count | (1 + inclusive prefix) << 32
    const unsigned int *over;    // overflow flag (the word after look[nb - 1])
    int cap;
};

// The fused path's view of the bucket words (c->bcnt holds 2 nb + 2 words for it).
inline FusedSort fused_sort_args(const nsg_ctx *c, int cap)
{
    return FusedSort{c->bidx, reinterpret_cast<unsigned long long *>(c->bcnt), c->bcnt + 2 * c->nb_total, cap};
}

__device__ __forceinline__ uint32_t fused_count(const FusedSort &fs, int b)
{
    return reinterpret_cast<const unsigned int *>(fs.look)[2 * b];
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}

__device__ __forceinline__ void st_relaxed_u32(unsigned int *p, unsigned int v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v));
}

// First sorted position of bucket b: the exclusive prefix of the bucket counts, by a
// decoupled look-back over the preceding buckets' words, fused into the kernel that
// consumes the sort (no scan kernel between the scatter and it).  Every count is
// final when the kernel starts, so no block ever waits on another: the block reads
// T predecessors at a time, nearest first, adds their counts down to the nearest one
// that has published its inclusive prefix (or past bucket 0, whose prefix is 0), adds
// that prefix and publishes its own.  The sum is exact in any order of publication.
//
// The first window is read when the block starts, beside the sort's own loads, and
// reduced inside the sort's first barrier (fused_block_minmax): per warp, the sum up
// to and including its nearest published word (flagged) and the sum of all its
// counts.  Blocks start in roughly index order and publish right after that barrier,
// so the nearest predecessors have usually published; only then does the block walk
// further windows (lookback_windows), e.g. in the first wave of the grid.
constexpr uint32_t kLookPub = 0x80000000u;   // warp partial: holds a published prefix

__device__ __forceinline__ unsigned long long lookback_word(const FusedSort &fs, int q)
{
    // a position before bucket 0 reads as published with prefix 0
    return q >= 0 ? ld_relaxed_u64(fs.look + q) : (1ull << 32);
}

// The warp's look-back partial for one window word per lane (lane l: bucket top-1-l
// of the warp's 32): low word = sum to the nearest published word (| kLookPub) or
// 0, high word = sum of all 32 counts.
__device__ __forceinline__ uint64_t lookback_partial(unsigned long long word)
{
    const uint32_t cq = (uint32_t)word, inc1 = (uint32_t)(word >> 32);
    const unsigned pub = __ballot_sync(0xffffffffu, inc1 != 0u);
    const int lane = threadIdx.x & 31;
    const int f = pub ? __ffs(pub) - 1 : 32;
    uint32_t part = lane < f ? cq : (lane == f ? inc1 - 1u : 0u);
    uint32_t all = cq;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        part += __shfl_xor_sync(0xffffffffu, part, o);
        all += __shfl_xor_sync(0xffffffffu, all, o);
    }
    return ((uint64_t)all << 32) | (pub ? (part | kLookPub) : 0u);
}

// Combines the warps' partials of one window (warp order = nearest first): adds to
// acc and returns whether a published prefix was reached.
template <int W>
__device__ __forceinline__ bool lookback_combine(const uint64_t *parts, uint32_t &acc)
{
#pragma unroll
    for (int i = 0; i < W; i++) {
        const uint64_t x = parts[i];
        if ((uint32_t)x & kLookPub) { acc += (uint32_t)x & ~kLookPub; return true; }
        acc += (uint32_t)(x >> 32);
    }
    return false;
}

// Further windows, from bucket top - 1 down, until a published prefix: adds to acc.
// All T threads call it (uniform); it uses its own barriers.
template <int T>
__device__ __noinline__ uint32_t lookback_windows(const FusedSort &fs, int top, uint32_t acc)
{
    constexpr int W = T / 32;
    __shared__ uint64_t s_part[2][W];
    const int w = threadIdx.x >> 5;
    for (int it = 0;; top -= T, it ^= 1) {
        const uint64_t pw = lookback_partial(lookback_word(fs, top - 1 - (int)threadIdx.x));
        if ((threadIdx.x & 31) == 0) s_part[it][w] = pw;
        __syncthreads();
        if (lookback_combine<W>(s_part[it], acc)) break;   // uniform; the next window writes the other half
    }
    return acc;
}

template <int T>
__device__ __forceinline__ void lookback_publish(const FusedSort &fs, int b, uint32_t acc, uint32_t m)
{
    if (threadIdx.x == 0) st_relaxed_u32(reinterpret_cast<unsigned int *>(fs.look + b) + 1, acc + m + 1u);
}

// The whole look-back for a block that sorts nothing (m = 0).
template <int T>
__device__ __forceinline__ void fused_lookback_empty(const FusedSort &fs, int b)
{
    lookback_publish<T>(fs, b, lookback_windows<T>(fs, b, 0u), 0u);
}

// An entry: its sort key in one word, and in the other the particle id (< 2^31),
// its source index and, in bit 63, whether the radius was -0.0 (whose key is that
// of +0.0).
constexpr uint64_t kNegZeroBit = 1ull << 63;

__device__ __forceinline__ int32_t entry_id(uint64_t e) { return (int32_t)((e >> 32) & 0x7fffffffu); }

__device__ __forceinline__ bool entry_less(uint64_t ka, uint64_t ea, uint64_t kb, uint64_t eb)
{
    return ka < kb || (ka == kb && ((ea >> 32) & 0x7fffffffu) < ((eb >> 32) & 0x7fffffffu));
}

// The radius of an entry from its key (radius_key inverted; -0.0 from the flag); a
// NaN radius, whose key keeps neither sign nor payload, is read again.
__device__ __forceinline__ double entry_radius(uint64_t k, uint64_t e, const double *__restrict__ r_src)
{
    if (k == ~0ull) return r_src[(uint32_t)e];
    uint64_t u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
    if (e & kNegZeroBit) u = 0x8000000000000000ull;
    return __longlong_as_double((long long)u);
}

// Block minimum and maximum of x (one tree, both words), and the first look-back
// window's combination (the warp partials `pw` in, the prefix sum so far out; returns
// whether it reached a published prefix).
template <int T>
__device__ __forceinline__ bool fused_block_minmax(uint64_t &mn, uint64_t &mx, uint64_t pw, uint32_t &acc,
                                                   uint64_t *red)
{
    constexpr int W = T / 32;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t y = __shfl_xor_sync(0xffffffffu, mn, o);
        const uint64_t z = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = y < mn ? y : mn;
        mx = z > mx ? z : mx;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { red[w] = mn; red[16 + w] = mx; red[32 + w] = pw; }
    __syncthreads();
    mn = red[0];
    mx = red[16];
#pragma unroll
    for (int i = 1; i < W; i++) {
        mn = red[i] < mn ? red[i] : mn;
        mx = red[16 + i] > mx ? red[16 + i] : mx;
    }
    acc = 0u;
    const bool found = lookback_combine<W>(red + 32, acc);
    __syncthreads();
    return found;
}

// Sorts the m entries of bucket b into sk[0..m) (keys) and se[0..m) (entries) by
// (key, id).  T threads (blockDim.x, at most 512), m <= cap <= T * kFusedItems,
// cap a power of two.  smem: fused_smem_bytes(cap).
// Also finds the bucket's first sorted position (the look-back above) and
// publishes its inclusive prefix; returns that position.
template <int T>
__device__ __forceinline__ uint32_t fused_bucket_sort(const FusedSort &fs, int b, uint32_t m,
                                                      const double *__restrict__ r_src,
                                                      const int32_t *__restrict__ id_src,
                                                      unsigned char *smem, uint64_t *&sk_out, uint64_t *&se_out)
{
    static_assert(T <= 512, "two reduction words per warp");
    constexpr int kBins = T * kFusedItems;               // = cap
    constexpr int kQB = fused_log2(kBins);
    uint64_t *sk = reinterpret_cast<uint64_t *>(smem);
    uint64_t *se = sk + fs.cap;
    uint32_t *bins = reinterpret_cast<uint32_t *>(se + fs.cap);            // kBins + 1
    uint64_t *red = reinterpret_cast<uint64_t *>(bins + kBins + 2);        // 8-aligned: kBins + 2 is even
    const int tid = threadIdx.x;
    sk_out = sk;
    se_out = se;

    // first look-back window: thread t reads bucket b-1-t, beside the loads below
    const unsigned long long lword = lookback_word(fs, b - 1 - tid);
    uint64_t key[kFusedItems], ent[kFusedItems];
    uint64_t kmin = ~0ull, kmax = 0ull;
    const uint32_t *src = fs.bidx + (size_t)b * fs.cap;
#pragma unroll
    for (int j = 0; j < kFusedItems; j++) {
        const uint32_t e = (uint32_t)(tid + j * T);
        if (e < m) {
            const uint32_t p = src[e];
            const double r = r_src[p];
            ent[j] = ((uint64_t)(uint32_t)id_src[p] << 32) | (uint64_t)p |
                     (dbits(r) == (long long)0x8000000000000000ull ? kNegZeroBit : 0ull);
            key[j] = radius_key(r);
            kmin = key[j] < kmin ? key[j] : kmin;
            kmax = key[j] > kmax ? key[j] : kmax;
        }
    }
    for (int q = tid; q <= kBins; q += T) bins[q] = 0u;
    uint32_t base;
    if (!fused_block_minmax<T>(kmin, kmax, lookback_partial(lword), base, red))
        base = lookback_windows<T>(fs, b - T, base);
    lookback_publish<T>(fs, b, base, m);
    const uint64_t span = kmax - kmin;
    const int sb = span ? 64 - __clzll((long long)span) : 0;
    const int qs = sb > kQB ? sb - kQB : 0;

    // counting sort on q: slot within the bin from a shared-memory atomic
    uint32_t qv[kFusedItems], slot[kFusedItems];
#pragma unroll
    for (int j = 0; j < kFusedItems; j++) {
        const uint32_t e = (uint32_t)(tid + j * T);
        if (e < m) {
            qv[j] = (uint32_t)((key[j] - kmin) >> qs);
            slot[j] = atomicAdd(&bins[qv[j]], 1u);
        }
    }
    __syncthreads();
    // exclusive scan of the bin counts in place; bins[kBins] = m
    {
        constexpr int per = kBins / T;
        uint32_t loc[per], s = 0;
#pragma unroll
        for (int k = 0; k < per; k++) { loc[k] = bins[tid * per + k]; s += loc[k]; }
        const int lane = tid & 31, w = tid >> 5;
        uint32_t x = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        uint32_t *wsum = reinterpret_cast<uint32_t *>(red);
        if (lane == 31) wsum[w] = x;
        __syncthreads();
        if (w == 0) {
            const uint32_t v = lane < T / 32 ? wsum[lane] : 0u;
            uint32_t z = v;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, z, o);
                if (lane >= o) z += y;
            }
            if (lane < T / 32) wsum[lane] = z - v;
        }
        __syncthreads();
        uint32_t run = wsum[w] + x - s;
#pragma unroll
        for (int k = 0; k < per; k++) { bins[tid * per + k] = run; run += loc[k]; }
        if (tid == 0) bins[kBins] = m;
        __syncthreads();
    }
    int big = 0;
    uint32_t lo[kFusedItems], cnt[kFusedItems];
#pragma unroll
    for (int j = 0; j < kFusedItems; j++) {
        const uint32_t e = (uint32_t)(tid + j * T);
        cnt[j] = 0u;
        if (e < m) {
            lo[j] = bins[qv[j]];
            cnt[j] = bins[qv[j] + 1] - lo[j];
            sk[lo[j] + slot[j]] = key[j];
            se[lo[j] + slot[j]] = ent[j];
            if (cnt[j] > (uint32_t)kFixupMax) big = 1;
        }
    }
    big = __syncthreads_or(big);
    if (!big) {
        // order each multi-entry bin by (key, id): rank among the bin's entries
        uint32_t fin[kFusedItems];
#pragma unroll
        for (int j = 0; j < kFusedItems; j++) {
            fin[j] = ~0u;
            if (cnt[j] > 1u) {
                uint32_t rank = 0;
                for (uint32_t t = 0; t < cnt[j]; t++)
                    rank += entry_less(sk[lo[j] + t], se[lo[j] + t], key[j], ent[j]) ? 1u : 0u;
                fin[j] = lo[j] + rank;
            }
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kFusedItems; j++) {
            if (fin[j] != ~0u) {
                sk[fin[j]] = key[j];
                se[fin[j]] = ent[j];
            }
        }
        __syncthreads();
        return base;
    }
    // bitonic sort of the whole bucket, padded to a power of two with entries that
    // order after every real one (largest key, id 2^31 - 1, above every id of a
    // state of at most 2^31 - 1 particles)
    uint32_t P = 1;
    while (P < m) P <<= 1;
    for (uint32_t e = m + tid; e < P; e += T) {
        sk[e] = ~0ull;
        se[e] = 0x7fffffff00000000ull;
    }
    __syncthreads();
    for (uint32_t k = 2; k <= P; k <<= 1) {
        for (uint32_t jj = k >> 1; jj > 0; jj >>= 1) {
            for (uint32_t i = tid; i < P; i += T) {
                const uint32_t l = i ^ jj;
                if (l > i) {
                    const bool up = (i & k) == 0;
                    const uint64_t ki = sk[i], ei = se[i], kl = sk[l], el = se[l];
                    const bool sw = up ? entry_less(kl, el, ki, ei) : entry_less(ki, ei, kl, el);
                    if (sw) { sk[i] = kl; se[i] = el; sk[l] = ki; se[l] = ei; }
                }
            }
            __syncthreads();
        }
    }
    return base;
}

// Halo of bucket b (the buckets of halo h are [bbase[h], bbase[h+1])).
__device__ __forceinline__ int halo_of_bucket(const Seg &sg, int b)
{
    if (sg.nseg <= 1) return 0;
    int lo = 0, hi = sg.nseg - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sg.bbase[mid] <= b) lo = mid; else hi = mid - 1;
    }
    return lo;
}

}  // namespace nsg
