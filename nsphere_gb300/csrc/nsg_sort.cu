// nsg_sort.cu -- radial sort of the resident state by (r, id) and the fused
// rank / enclosed-mass / force pass.
//
// Replaces sort_particles (nsphere.c:8605-8665, quadsort of the five columns by
// r) plus the inverse_map rebuild (nsphere.c:5789-5794).  The enclosed mass of
// the reference is the sorted rank, M_i = (i/N) M (nsphere.c:513); the pass after
// the sort writes, per sorted position, the force at the step start
// gnum_i/r^2 + ell^2/r^3 (nsphere.c:502-535), the inverse map and the energy
// partial sums.
//
// Sort algorithm (general path): the permutation is seeded in id order (ids are a
// permutation of 0..n-1), then an LSD radix sort over the 64-bit order-preserving
// radius key, 8 bits per pass, stable.  Stability on an id-ordered start gives the
// (r, id) total order.  Each pass: per-tile digit counts -> per-digit scan ->
// stable warp-level ranking (match.any) and scatter.  No kernel waits on another
// block, so no spin loops.
#include "nsg_fused.cuh"

namespace nsg {

// Seeds the sort: keys[id] = key(r), vals[id] = source index.  Marks NaN radii.
__global__ void k_seed_keys(const double *__restrict__ r, const int32_t *__restrict__ id,
                            int64_t n, uint64_t *__restrict__ keys, uint32_t *__restrict__ vals,
                            DevCounters *ctr)
{
    if (!ctr->need_fallback) return;
    bool nan_seen = false;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        double rk = r[k];
        int32_t j = id[k];
        nan_seen |= (rk != rk);
        keys[j] = radius_key(rk);
        vals[j] = (uint32_t)k;
    }
    if (nan_seen) atomicOr(&ctr->status, NSG_ST_NAN);
}

// Digit of one pass: 8 key bits at `shift` >= 0, or for shift = -1, -2 the low / high
// byte of the halo of the element's source position (the passes that group an
// ensemble by halo after the key passes).
__device__ __forceinline__ unsigned radix_digit(uint64_t key, uint32_t val, int shift, const Seg &sg)
{
    if (shift >= 0) return (unsigned)(key >> shift) & (kRadixBuckets - 1);
    return ((unsigned)seg_of(sg, val) >> ((-shift - 1) * 8)) & (kRadixBuckets - 1);
}

// Per-tile histogram of one digit.  counts is digit-major: counts[d * ntiles + t].
__global__ void __launch_bounds__(kRadixThreads)
k_tile_hist(const uint64_t *__restrict__ keys, const uint32_t *__restrict__ vals, int64_t n, int shift,
            int ntiles, uint32_t *__restrict__ counts, const DevCounters *__restrict__ ctr, Seg sg)
{
    if (!ctr->need_fallback) return;
    __shared__ uint32_t h[kRadixBuckets];
    for (int d = threadIdx.x; d < kRadixBuckets; d += blockDim.x) h[d] = 0;
    __syncthreads();
    int64_t base = (int64_t)blockIdx.x * kRadixTile;
#pragma unroll 4
    for (int j = 0; j < kRadixItems; j++) {
        int64_t idx = base + j * kRadixThreads + threadIdx.x;
        if (idx < n) atomicAdd(&h[radix_digit(keys[idx], vals[idx], shift, sg)], 1u);
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixBuckets; d += blockDim.x)
        counts[(int64_t)d * ntiles + blockIdx.x] = h[d];
}

// Block-wide exclusive scan of one value per thread (blockDim.x == 1024).
__device__ __forceinline__ uint32_t block_excl_scan_1024(uint32_t v, uint32_t *warp_tot,
                                                         uint32_t *total)
{
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = warp_tot[lane];
        uint32_t s = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        warp_tot[lane] = s - t;
        if (lane == 31) *total = s;
    }
    __syncthreads();
    uint32_t r = warp_tot[w] + x - v;
    __syncthreads();
    return r;
}

// Sum of each digit's row of tile counts.  One block per digit.
__global__ void __launch_bounds__(1024)
k_digit_totals(const uint32_t *__restrict__ counts, int ntiles, uint32_t *__restrict__ tot,
               const DevCounters *__restrict__ ctr)
{
    if (!ctr->need_fallback) return;
    __shared__ uint32_t wsum[32];
    const uint32_t *row = counts + (int64_t)blockIdx.x * ntiles;
    uint32_t s = 0;
    for (int t = threadIdx.x; t < ntiles; t += blockDim.x) s += row[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        s = wsum[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (threadIdx.x == 0) tot[blockIdx.x] = s;
    }
}

// Turns each digit's row into global exclusive offsets: base(digit) + prefix over
// tiles.  One block per digit.
__global__ void __launch_bounds__(1024)
k_digit_scan(uint32_t *__restrict__ counts, int ntiles, const uint32_t *__restrict__ tot,
             const DevCounters *__restrict__ ctr)
{
    if (!ctr->need_fallback) return;
    __shared__ uint32_t warp_tot[32];
    __shared__ uint32_t total;
    __shared__ uint32_t base_s;
    if (threadIdx.x == 0) {
        uint32_t b = 0;
        for (int d = 0; d < (int)blockIdx.x; d++) b += tot[d];
        base_s = b;
    }
    __syncthreads();
    uint32_t carry = base_s;
    uint32_t *row = counts + (int64_t)blockIdx.x * ntiles;
    for (int t0 = 0; t0 < ntiles; t0 += 1024) {
        int t = t0 + threadIdx.x;
        uint32_t v = (t < ntiles) ? row[t] : 0u;
        uint32_t ex = block_excl_scan_1024(v, warp_tot, &total);
        if (t < ntiles) row[t] = carry + ex;
        carry += total;
        __syncthreads();
    }
}

// Stable ranking and scatter of one tile for one digit.  Warp w of the block owns
// 512 consecutive keys; item j of lane l is key base + j*32 + l, so walking j and
// then lanes visits the keys in input order and the match.any ranks are stable.
__global__ void __launch_bounds__(kRadixThreads)
k_scatter(const uint64_t *__restrict__ keys_in, const uint32_t *__restrict__ vals_in,
          uint64_t *__restrict__ keys_out, uint32_t *__restrict__ vals_out, int64_t n,
          int shift, int ntiles, const uint32_t *__restrict__ offsets,
          const DevCounters *__restrict__ ctr, Seg sg)
{
    if (!ctr->need_fallback) return;
    constexpr int W = kRadixThreads / 32;
    __shared__ uint32_t whist[W][kRadixBuckets];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < W * kRadixBuckets; d += blockDim.x) (&whist[0][0])[d] = 0;
    __syncthreads();

    const int64_t base = (int64_t)blockIdx.x * kRadixTile + (int64_t)w * (kRadixItems * 32);
    const unsigned lt = lanemask_lt();
    uint64_t k[kRadixItems];
    uint32_t v[kRadixItems];
    uint32_t rank[kRadixItems];
    uint32_t dig[kRadixItems];
#pragma unroll
    for (int j = 0; j < kRadixItems; j++) {
        int64_t idx = base + j * 32 + lane;
        bool ok = idx < n;
        k[j] = ok ? keys_in[idx] : 0ull;
        v[j] = ok ? vals_in[idx] : 0u;
        dig[j] = ok ? radix_digit(k[j], v[j], shift, sg) : (unsigned)kRadixBuckets;
    }
#pragma unroll
    for (int j = 0; j < kRadixItems; j++) {
        unsigned d = dig[j];
        unsigned peers = __match_any_sync(0xffffffffu, d);
        uint32_t cnt = 0;
        if (d < kRadixBuckets) cnt = whist[w][d];
        rank[j] = cnt + __popc(peers & lt);
        __syncwarp();
        if (d < kRadixBuckets && lane == __ffs(peers) - 1) whist[w][d] = cnt + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadixBuckets; d += blockDim.x) {
        uint32_t run = offsets[(int64_t)d * ntiles + blockIdx.x];
#pragma unroll
        for (int ww = 0; ww < W; ww++) {
            uint32_t t = whist[ww][d];
            whist[ww][d] = run;
            run += t;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kRadixItems; j++) {
        unsigned d = dig[j];
        if (d < kRadixBuckets) {
            uint32_t pos = whist[w][d] + rank[j];
            keys_out[pos] = k[j];
            vals_out[pos] = v[j];
        }
    }
}

// Gathers the state into sorted order and computes, per sorted position p, the
// acceleration at the step start a0 = gnum/r^2 + ell^2/r^3 with the force numerator
// of the particle's rank within its halo (nsphere.c:502-535), the inverse map
// (nsphere.c:5789-5794) and the next sort's splitters.  KICK applies the second
// half-kick of the fixed-step body with the new rank, v += 0.5*a0*dt
// (nsphere.c:5520-5531), in the same pass.
template <bool AUX, bool KICK>
__global__ void __launch_bounds__(256)
k_gather_rank_force(const uint32_t *__restrict__ perm, int64_t n,
                    const double *__restrict__ r0, const double *__restrict__ v0,
                    const double *__restrict__ l0, const int32_t *__restrict__ id0,
                    const double *__restrict__ x0,
                    double *__restrict__ r1, double *__restrict__ v1, double *__restrict__ l1,
                    int32_t *__restrict__ id1, double *__restrict__ x1,
                    double *__restrict__ a0, int32_t *__restrict__ inv, uint64_t *__restrict__ split,
                    double G, double M, double dt, const DevCounters *__restrict__ ctr, Seg sg,
                    const unsigned *__restrict__ run_if)
{
    if (run_if && *run_if == 0u) return;   // fallback consumer: the fused kernel did the work
    const double Mpt = ctr->point_mass;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        const Local L = local_of(sg, p, n);
        uint32_t s = perm[p];
        double r = r0[s], v = v0[s], l = l0[s];
        int32_t idv = id0[s];
        double gn = gnum_of(L.i, L.n, G, M, Mpt);
        double acc = acc_leap(r, gn, dmul(l, l));
        if (KICK) v = dadd(v, dmul(half_exact(acc), dt));
        r1[p] = r;
        v1[p] = v;
        l1[p] = l;
        id1[p] = idv;
        if (AUX) x1[p] = x0[s];
        inv[idv] = (int32_t)p;
        a0[p] = acc;
        write_splitter(split, sg, L, r);
    }
}

// The same pass with the near-sorted sort done in the block (nsg_fused.cuh): block b
// sorts bucket b and writes its sorted positions off[b] .. off[b] + cnt[b] - 1
// (off[b] from the look-back over the counts, nsg_fused.cuh).
template <bool AUX, bool KICK, int T>
__global__ void __launch_bounds__(T, T == 128 ? 8 : (T == 256 ? 4 : 2))
k_fused_rank_force(FusedSort fs, int64_t n,
                   const double *__restrict__ r0, const double *__restrict__ v0,
                   const double *__restrict__ l0, const int32_t *__restrict__ id0,
                   const double *__restrict__ x0,
                   double *__restrict__ r1, double *__restrict__ v1, double *__restrict__ l1,
                   int32_t *__restrict__ id1, double *__restrict__ x1,
                   double *__restrict__ a0, int32_t *__restrict__ inv, uint64_t *__restrict__ split,
                   double G, double M, double dt, DevCounters *__restrict__ ctr, Seg sg)
{
    const unsigned over = *fs.over;
    if (blockIdx.x == 0 && threadIdx.x == 0) ctr->need_fallback = over;   // read after this kernel
    if (over) return;
    const int b = blockIdx.x;
    const uint32_t m = fused_count(fs, b);
    if (m == 0u) {
        fused_lookback_empty<T>(fs, b);
        return;
    }
    extern __shared__ __align__(16) unsigned char fsm[];
    uint64_t *sr, *sv;
    const int64_t base = fused_bucket_sort<T>(fs, b, m, r0, id0, fsm, sr, sv);
    const double Mpt = ctr->point_mass;
    const int h = halo_of_bucket(sg, b);
    const int64_t hs = sg.nseg <= 1 ? 0 : sg.start[h];
    const int64_t hn = sg.nseg <= 1 ? n : sg.start[h + 1] - hs;
    for (uint32_t j = threadIdx.x; j < m; j += T) {
        const int64_t p = base + j;
        const Local L{p - hs, hn, h};
        const uint64_t e = sv[j];
        const uint32_t s = (uint32_t)e;
        const int32_t idv = entry_id(e);
        const double r = entry_radius(sr[j], e, r0);
        double v = v0[s];
        const double l = l0[s];
        const double gn = gnum_of(L.i, L.n, G, M, Mpt);
        const double acc = acc_leap(r, gn, dmul(l, l));
        if (KICK) v = dadd(v, dmul(half_exact(acc), dt));
        r1[p] = r;
        v1[p] = v;
        l1[p] = l;
        id1[p] = idv;
        if (AUX) x1[p] = x0[s];
        inv[idv] = (int32_t)p;
        a0[p] = acc;
        write_splitter(split, sg, L, r);
    }
}

__device__ __forceinline__ void energy_terms(double rr, double vv, double ll, const Local &L, double G,
                                             double M, double Mpt, double &ek, double &ew)
{
    const double m = M / (double)L.n;
    const double gn = gnum_of(L.i, L.n, G, M, Mpt);
    ek += 0.5 * m * (vv * vv + (ll * ll) / (rr * rr));
    ew += m * gn / rr;
}

// Block sum of two doubles in a fixed tree order; thread 0 gets the result.
__device__ __forceinline__ void block_sum2(double &a, double &b)
{
    __shared__ double sk[32], sw[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) { sk[w] = a; sw[w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) { x += sk[i]; y += sw[i]; }
        a = x;
        b = y;
    }
}

// Energy partial sums of a sorted single halo: K = sum 1/2 m (v^2 + ell^2/r^2),
// W = sum m gnum_i / r_i.  Fixed grid and tree order: deterministic.
__global__ void __launch_bounds__(256)
k_energy(const double *__restrict__ r, const double *__restrict__ v, const double *__restrict__ l,
         int64_t n, double G, double M, const DevCounters *__restrict__ ctr, double *__restrict__ red_part)
{
    const double Mpt = ctr->point_mass;
    double ek = 0.0, ew = 0.0;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x)
        energy_terms(r[p], v[p], l[p], Local{p, n, 0}, G, M, Mpt, ek, ew);
    block_sum2(ek, ew);
    if (threadIdx.x == 0) {
        red_part[blockIdx.x] = ek;
        red_part[kReduceBlocks + blockIdx.x] = ew;
    }
}

// Energies of an ensemble: one block per halo, deterministic order.
__global__ void __launch_bounds__(256)
k_energy_seg(const double *__restrict__ r, const double *__restrict__ v, const double *__restrict__ l,
             int64_t n, double G, double M, const DevCounters *__restrict__ ctr, Seg sg,
             double *__restrict__ seg_energy)
{
    const double Mpt = ctr->point_mass;
    const int h = blockIdx.x;
    const int64_t st = sg.start[h], nh = sg.start[h + 1] - st;
    double ek = 0.0, ew = 0.0;
    for (int64_t q = threadIdx.x; q < nh; q += blockDim.x)
        energy_terms(r[st + q], v[st + q], l[st + q], Local{q, nh, h}, G, M, Mpt, ek, ew);
    block_sum2(ek, ew);
    if (threadIdx.x == 0) {
        seg_energy[2 * h] = ek;
        seg_energy[2 * h + 1] = ew;
    }
}

__global__ void k_finalize_energy(const double *__restrict__ kpart, const double *__restrict__ wpart,
                                  int nblk, int stride, DevCounters *ctr)
{
    double a = 0.0, b = 0.0;
    for (int i = threadIdx.x; i < nblk; i += blockDim.x) { a += kpart[i * stride]; b += wpart[i * stride]; }
    block_sum2(a, b);
    if (threadIdx.x == 0) {
        ctr->energy[0] = a;
        ctr->energy[1] = b;
    }
}

// Sorts the live copy by (halo, r, id); leaves the permutation in c->perm.
// Seed keys and the radix passes on stream s; returns the buffer that ends with the
// permutation.  Every kernel returns at once unless ctr->need_fallback is set.
static int launch_radix(nsg_ctx *c, cudaStream_t s, int *kb_out)
{
    const int64_t n = c->n;
    const int src = c->cur;
    const int ntiles = (int)((n + kRadixTile - 1) / kRadixTile);
    const Seg sg = seg_table(c);
    {
        ProfScope ps(c, "sort_seed", (double)n * (8 + 4 + 8 + 4), s);
        k_seed_keys<<<grid_for(c, n, 256), 256, 0, s>>>(c->r[src], c->id[src], n, c->keys[0],
                                                         c->vals[0], c->ctr);
    }
    // 8 passes over the radius key, then (ensembles) 2 stable passes over the halo
    // index; an even pass count leaves the permutation in vals[0], where the bucket
    // path writes it too
    const int npass = 8 + (c->nseg > 1 ? 2 : 0);
    int kb = 0;
    {
        ProfScope ps(c, "sort_radix", (double)n * npass * (8 + 12 + 12), s);
        for (int pass = 0; pass < npass; pass++) {
            const int shift = pass < 8 ? pass * kRadixBits : -(pass - 8 + 1);
            k_tile_hist<<<ntiles, kRadixThreads, 0, s>>>(c->keys[kb], c->vals[kb], n, shift, ntiles,
                                                         c->tile_counts, c->ctr, sg);
            k_digit_totals<<<kRadixBuckets, 1024, 0, s>>>(c->tile_counts, ntiles, c->digit_tot, c->ctr);
            k_digit_scan<<<kRadixBuckets, 1024, 0, s>>>(c->tile_counts, ntiles, c->digit_tot, c->ctr);
            k_scatter<<<ntiles, kRadixThreads, 0, s>>>(c->keys[kb], c->vals[kb], c->keys[1 - kb],
                                                       c->vals[1 - kb], n, shift, ntiles,
                                                       c->tile_counts, c->ctr, sg);
            kb = 1 - kb;
        }
    }
    *kb_out = kb;
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "sort kernels");
}

__global__ void k_radix_cond(cudaGraphConditionalHandle h, const DevCounters *__restrict__ ctr)
{
    if (threadIdx.x == 0) cudaGraphSetConditional(h, ctr->need_fallback ? 1u : 0u);
}

int radix_fallback(nsg_ctx *c, cudaStream_t s, int (*tail)(nsg_ctx *, cudaStream_t, const unsigned *, void *),
                   void *arg)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, nullptr, nullptr, nullptr);
    if (e != cudaSuccess) return cuda_err(c, e, "capture status");
    int kb = 0;
    const int npass = 8 + (c->nseg > 1 ? 2 : 0);
    if (cs != cudaStreamCaptureStatusActive || !c->cond_nodes) {
        if (cs != cudaStreamCaptureStatusActive && c->gate_fallback) {
            // An eager step inside a call that waits for the step anyway: read whether
            // the near-sorted path overflowed and launch the radix sort and its
            // consumer only then (otherwise their 34-42 launches each return at once).
            e = cudaMemcpyAsync(&c->h_ctr->need_fallback, &c->ctr->need_fallback, sizeof(unsigned),
                                cudaMemcpyDeviceToHost, s);
            if (e == cudaSuccess) e = cudaStreamSynchronize(s);
            if (e != cudaSuccess) return cuda_err(c, e, "fallback flag");
            if (c->h_ctr->need_fallback == 0u) {
                c->perm = c->vals[0];   // where the near-sorted path leaves the permutation
                return NSG_OK;
            }
        }
        if (int rc = launch_radix(c, s, &kb)) return rc;
        c->launches += 1 + npass * 4;
        c->perm = c->vals[kb];
        if (tail)
            if (int rc = tail(c, s, &c->ctr->need_fallback, arg)) return rc;
        return NSG_OK;
    }
    // In a captured step the radix kernels (and the consumer that goes with them) sit
    // in the body of a conditional node that a one-thread kernel opens only when the
    // near-sorted path overflowed: the 33-41 launches that would return at once cost
    // nothing.
    cudaGraphConditionalHandle h;
    e = cudaGraphConditionalHandleCreate(&h, g, 0, 0);
    if (e != cudaSuccess) return cuda_err(c, e, "conditional handle");
    k_radix_cond<<<1, 32, 0, s>>>(h, c->ctr);
    c->launches += 1;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(s, &cs, nullptr, &g, &deps, nullptr, &nd);
    if (e != cudaSuccess) return cuda_err(c, e, "capture dependencies");
    cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeIf;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &cp);
    if (e != cudaSuccess) return cuda_err(c, e, "conditional node");
    e = cudaStreamBeginCaptureToGraph(c->body, cp.conditional.phGraph_out[0], nullptr, nullptr, 0,
                                      cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return cuda_err(c, e, "conditional body capture");
    int rc = launch_radix(c, c->body, &kb);
    c->perm = c->vals[kb];
    if (!rc && tail) rc = tail(c, c->body, nullptr, arg);
    cudaGraph_t bg = nullptr;
    e = cudaStreamEndCapture(c->body, &bg);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_err(c, e, "conditional body capture");
    e = cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    if (e != cudaSuccess) return cuda_err(c, e, "capture dependencies");
    return NSG_OK;
}

int sort_perm(nsg_ctx *c)
{
    cudaStream_t s = c->stream;
    // near-sorted fast path when the array is in the order of a previous sort;
    // the radix kernels below run only if it overflowed (or it was not used)
    if (c->split_valid && c->p.sort_mode == 0) {
        if (int rc = bucket_sort_perm(c)) return rc;
    } else {
        // any non-zero value selects the radix path (bytes set to 0x01)
        cudaError_t e = cudaMemsetAsync(&c->ctr->need_fallback, 1, sizeof(unsigned), s);
        if (e != cudaSuccess) return cuda_err(c, e, "fallback flag");
    }
    return radix_fallback(c, s, nullptr, nullptr);
}

// The two-kernel consumer: k_gather_rank_force through c->perm on stream s (run_if:
// return at once unless *run_if is set).
static int launch_gather(nsg_ctx *c, bool kick, cudaStream_t s, const unsigned *run_if)
{
    const int64_t n = c->n;
    const int src = c->cur, dst = 1 - c->cur;
    const Seg sg = seg_table(c);
    ProfScope ps(c, run_if ? (kick ? "gather_kick_fallback" : "rank_force_fallback") : (kick ? "gather_kick" : "rank_force"),
                 (double)n * (4 + 28 + 28 + 8 + 4 + (c->p.carry_aux ? 16 : 0)), s);
    const int grid = grid_for(c, n, 256, 8);
#define NSG_GATHER(AUXV, KICKV)                                                                   \
    k_gather_rank_force<AUXV, KICKV><<<grid, 256, 0, s>>>(                                        \
        c->perm, n, c->r[src], c->vr[src], c->ell[src], c->id[src], c->aux[src], c->r[dst],      \
        c->vr[dst], c->ell[dst], c->id[dst], c->aux[dst], c->a0, c->inv, c->split, c->p.G,       \
        c->p.M_total, c->p.dt, c->ctr, sg, run_if)
    if (c->p.carry_aux) { if (kick) NSG_GATHER(true, true); else NSG_GATHER(true, false); }
    else { if (kick) NSG_GATHER(false, true); else NSG_GATHER(false, false); }
#undef NSG_GATHER
    c->launches += 1;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "gather kernel");
}

static int gather_tail(nsg_ctx *c, cudaStream_t s, const unsigned *run_if, void *arg)
{
    return launch_gather(c, *static_cast<const bool *>(arg), s, run_if);
}

template <int T>
static void launch_fused_force(nsg_ctx *c, bool kick, cudaStream_t s)
{
    const int64_t n = c->n;
    const int src = c->cur, dst = 1 - c->cur;
    const int cap = fused_cap(c);
    const FusedSort fs = fused_sort_args(c, cap);
    const size_t sm = fused_smem_bytes(cap);
    const int nb = (int)c->nb_total;
#define NSG_FUSED(AUXV, KICKV)                                                                          \
    k_fused_rank_force<AUXV, KICKV, T><<<nb, T, sm, s>>>(                                               \
        fs, n, c->r[src], c->vr[src], c->ell[src], c->id[src], c->aux[src], c->r[dst], c->vr[dst],      \
        c->ell[dst], c->id[dst], c->aux[dst], c->a0, c->inv, c->split, c->p.G, c->p.M_total, c->p.dt,  \
        c->ctr, seg_table(c))
    if (c->p.carry_aux) { if (kick) NSG_FUSED(true, true); else NSG_FUSED(true, false); }
    else { if (kick) NSG_FUSED(false, true); else NSG_FUSED(false, false); }
#undef NSG_FUSED
}

static int sort_gather(nsg_ctx *c, bool kick)
{
    const int64_t n = c->n;
    cudaStream_t s = c->stream;
    if (use_fused(c)) {
        if (int rc = bucket_fused_prepare(c, s)) return rc;
        {
            // algorithmic bytes: index 4, r id 12, v ell 16, write r v ell id 28, a0 8, inv 4
            ProfScope ps(c, kick ? "fused_kick" : "fused_force", (double)n * (4 + 12 + 16 + 28 + 8 + 4 +
                                                                               (c->p.carry_aux ? 16 : 0)), s);
            if (fused_cap(c) == 4096) launch_fused_force<512>(c, kick, s);
            else if (fused_cap(c) == 2048) launch_fused_force<256>(c, kick, s);
            else launch_fused_force<128>(c, kick, s);
            c->launches += 1;
        }
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return cuda_err(c, e, "fused sort kernel");
        bool k = kick;
        if (int rc = radix_fallback(c, s, gather_tail, &k)) return rc;
    } else {
        if (int rc = sort_perm(c)) return rc;
        if (int rc = launch_gather(c, kick, s, nullptr)) return rc;
    }
    c->cur = 1 - c->cur;
    c->state_epoch++;
    c->sorted = true;
    c->inv_valid = true;
    c->split_valid = true;
    return NSG_OK;
}

int sort_state(nsg_ctx *c)
{
    return sort_gather(c, false);
}

int sort_state_kick(nsg_ctx *c)
{
    return sort_gather(c, true);
}

int fused_force_setup(nsg_ctx *c)
{
    cudaError_t e = cudaSuccess;
#define NSG_ATTR(AUXV, KICKV, TV)                                                                       \
    if (e == cudaSuccess)                                                                               \
        e = cudaFuncSetAttribute(k_fused_rank_force<AUXV, KICKV, TV>,                                    \
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fused_smem_bytes(2 * TV * 4));
    NSG_ATTR(false, false, 128) NSG_ATTR(false, true, 128) NSG_ATTR(true, false, 128) NSG_ATTR(true, true, 128)
    NSG_ATTR(false, false, 256) NSG_ATTR(false, true, 256) NSG_ATTR(true, false, 256) NSG_ATTR(true, true, 256)
    NSG_ATTR(false, false, 512) NSG_ATTR(false, true, 512) NSG_ATTR(true, false, 512) NSG_ATTR(true, true, 512)
#undef NSG_ATTR
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "fused sort attributes");
}

int compute_energy(nsg_ctx *c)
{
    const int s = c->cur;
    if (c->nseg <= 1) {
        k_energy<<<kReduceBlocks, 256, 0, c->stream>>>(c->r[s], c->vr[s], c->ell[s], c->n, c->p.G,
                                                       c->p.M_total, c->ctr, c->red_part);
        k_finalize_energy<<<1, 1024, 0, c->stream>>>(c->red_part, c->red_part + kReduceBlocks,
                                                     kReduceBlocks, 1, c->ctr);
    } else {
        k_energy_seg<<<c->nseg, 256, 0, c->stream>>>(c->r[s], c->vr[s], c->ell[s], c->n, c->p.G, c->p.M_total,
                                                      c->ctr, seg_table(c), c->seg_energy);
        k_finalize_energy<<<1, 1024, 0, c->stream>>>(c->seg_energy, c->seg_energy + 1, c->nseg, 2, c->ctr);
    }
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "energy kernels");
}

}  // namespace nsg
