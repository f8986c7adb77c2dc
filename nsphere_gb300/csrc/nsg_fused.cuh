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
//   4. hands sorted position j of the bucket (global position off[b] + j) with its
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
// Layout: keys [cap] | entries [cap] | bin offsets [cap + 1] (+1 pad) | 32 reduction
// words.
__host__ __device__ constexpr size_t fused_smem_bytes(int cap)
{
    return (size_t)cap * 16 + (size_t)(cap + 2) * 4 + 32 * 8;
}

__host__ __device__ constexpr int fused_log2(int x) { return x <= 1 ? 0 : 1 + fused_log2(x >> 1); }

struct FusedSort {
    const uint32_t *bidx;      // [nb * cap] source indices per bucket
    const unsigned int *cnt;   // [nb] entries per bucket
    const unsigned int *off;   // [nb] first sorted position of each bucket (exclusive scan)
    int cap;
};

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

// Block minimum and maximum of x (one tree, both words).
__device__ __forceinline__ void fused_block_minmax(uint64_t &mn, uint64_t &mx, uint64_t *red)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t y = __shfl_xor_sync(0xffffffffu, mn, o);
        const uint64_t z = __shfl_xor_sync(0xffffffffu, mx, o);
        mn = y < mn ? y : mn;
        mx = z > mx ? z : mx;
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    if (lane == 0) { red[w] = mn; red[16 + w] = mx; }
    __syncthreads();
    mn = red[0];
    mx = red[16];
    for (int i = 1; i < nw; i++) {
        mn = red[i] < mn ? red[i] : mn;
        mx = red[16 + i] > mx ? red[16 + i] : mx;
    }
    __syncthreads();
}

// Sorts the m entries of bucket b into sk[0..m) (keys) and se[0..m) (entries) by
// (key, id).  T threads (blockDim.x, at most 512), m <= cap <= T * kFusedItems,
// cap a power of two.  smem: fused_smem_bytes(cap).
template <int T>
__device__ __forceinline__ void fused_bucket_sort(const FusedSort &fs, int b, uint32_t m,
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
    fused_block_minmax(kmin, kmax, red);
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
        return;
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
