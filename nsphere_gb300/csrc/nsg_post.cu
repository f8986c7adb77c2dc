// nsg_post.cu -- per-snapshot quantities of the reference's post-processing computed
// on the resident state (nsphere.c:7697-7846): the potential of the particle
// distribution at each sorted radius,
//     Psi_A(r_i) = G ( M_i / r_i + dM sum_{j > i} 1 / r_j ),  M_i = (i + 1) dM,
// its central value Psi_A(0) = G dM sum_j 1 / r_j, and each particle's energy
// E_i = Psi_A(r_i) - ell_i^2 / (2 r_i^2) - v_i^2 / 2, with dM = M_total / N.
// The reference sums 1/r sequentially from the outermost particle inwards; here the
// suffix sums are a three-pass parallel scan (block sums, one scan of the block sums,
// block-local suffix scans), so the results agree with the reference to the rounding
// of the two summation orders (the terms are all positive: a relative difference of
// order 1e-13 at N = 1e5).
#include "nsg_internal.cuh"

namespace nsg {

constexpr int kPostThreads = 256, kPostItems = 4, kPostTile = kPostThreads * kPostItems;

__device__ __forceinline__ double block_sum_d(double v, double *sh)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    return t;   // valid in thread 0
}

__global__ void __launch_bounds__(kPostThreads) k_post_tile_sums(const double *__restrict__ r, int64_t n,
                                                                 double *__restrict__ tile_sum)
{
    __shared__ double sh[32];
    const int64_t base = (int64_t)blockIdx.x * kPostTile;
    double s = 0.0;
    for (int k = 0; k < kPostItems; k++) {
        const int64_t i = base + k * kPostThreads + threadIdx.x;
        if (i < n) s += 1.0 / r[i];
    }
    s = block_sum_d(s, sh);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = s;
}

// In place: tile_sum[t] <- sum of tiles t+1 .. ntiles-1 (exclusive suffix scan); the
// total goes to *total.  One block of 1024 threads, each owning a contiguous run.
__global__ void __launch_bounds__(1024) k_post_scan_tiles(double *tile_sum, int64_t ntiles, double *total)
{
    __shared__ double sh[1024];
    const int t = threadIdx.x;
    const int64_t per = (ntiles + 1023) / 1024;
    const int64_t lo = t * per < ntiles ? t * per : ntiles, hi = lo + per < ntiles ? lo + per : ntiles;
    double s = 0.0;
    for (int64_t j = lo; j < hi; j++) s += tile_sum[j];
    sh[t] = s;
    __syncthreads();
    // suffix sums of the 1024 run totals (Hillis-Steele from the right)
    for (int o = 1; o < 1024; o <<= 1) {
        const double v = (t + o < 1024) ? sh[t + o] : 0.0;
        __syncthreads();
        sh[t] += v;
        __syncthreads();
    }
    double run = (t + 1 < 1024) ? sh[t + 1] : 0.0;     // sum of the runs after this one
    if (t == 0) *total = sh[0];
    for (int64_t j = hi - 1; j >= lo; j--) {
        const double v = tile_sum[j];
        tile_sum[j] = run;
        run += v;
    }
}

__global__ void __launch_bounds__(kPostThreads) k_post_energy(const double *__restrict__ r,
                                                              const double *__restrict__ v,
                                                              const double *__restrict__ l, int64_t n,
                                                              const double *__restrict__ tile_after, double G,
                                                              double dM, double *__restrict__ psi,
                                                              double *__restrict__ E)
{
    constexpr int kSeg = kPostTile / 32;
    __shared__ double suf[kPostTile];     // suffix sums of 1/r inside each 32-element segment
    __shared__ double after[32];          // sum of 1/r over everything right of each segment
    const int64_t base = (int64_t)blockIdx.x * kPostTile;
    for (int k = threadIdx.x; k < kPostTile; k += kPostThreads) {
        const int64_t i = base + k;
        suf[k] = i < n ? 1.0 / r[i] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int lo = threadIdx.x * kSeg;
        double s = 0.0;
        for (int k = lo + kSeg - 1; k >= lo; k--) {
            s += suf[k];
            suf[k] = s;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double acc = tile_after[blockIdx.x];
        for (int g = 31; g >= 0; g--) {
            after[g] = acc;
            acc += suf[g * kSeg];
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < kPostTile; k += kPostThreads) {
        const int64_t i = base + k;
        if (i >= n) continue;
        const int g = k / kSeg;
        const double within = (k + 1 < (g + 1) * kSeg) ? suf[k + 1] : 0.0;   // j > i in the segment
        const double S = within + after[g];
        const double ri = r[i];
        const double Mi = (double)(i + 1) * dM;
        const double p = G * (Mi / ri + dM * S);
        psi[i] = p;
        const double li = l[i], vi = v[i];
        E[i] = p - li * li / (2.0 * ri * ri) - 0.5 * vi * vi;
    }
}

// Psi_A at each sorted radius into psi[0..n) (and the energies into E) for a sorted
// radius array r with velocities v, ell; the total of 1/r goes to *total (device).
// tile: ceil(n / kPostTile) doubles of scratch.
int post_psi_sorted(nsg_ctx *c, const double *r, const double *v, const double *l, int64_t n, double *psi,
                    double *E, double *tile, double *total)
{
    const int64_t ntiles = (n + kPostTile - 1) / kPostTile;
    cudaStream_t s = c->stream;
    k_post_tile_sums<<<(unsigned)ntiles, kPostThreads, 0, s>>>(r, n, tile);
    k_post_scan_tiles<<<1, 1024, 0, s>>>(tile, ntiles, total);
    k_post_energy<<<(unsigned)ntiles, kPostThreads, 0, s>>>(r, v, l, n, tile, c->p.G, c->p.M_total / (double)n,
                                                            psi, E);
    c->launches += 3;
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "potential");
}

int64_t post_tiles(int64_t n) { return (n + kPostTile - 1) / kPostTile; }

}  // namespace nsg

using namespace nsg;

extern "C" int nsg_potential(nsg_ctx *c, double *psi, double *E, double *psi0)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (c->nseg > 1) return set_err(c, NSG_EINVAL, "the distribution potential is defined for one halo");
    if (!c->sorted)
        if (int rc = sort_state(c)) return rc;
    const int64_t n = c->n, ntiles = (n + kPostTile - 1) / kPostTile;
    const int k = c->cur;
    double *d = nullptr;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMallocAsync((void **)&d, (size_t)(2 * n + ntiles + 1) * sizeof(double), s);
    if (e != cudaSuccess) return cuda_err(c, e, "potential");
    double *d_psi = d, *d_E = d + n, *d_tile = d + 2 * n, *d_total = d + 2 * n + ntiles;
    k_post_tile_sums<<<(unsigned)ntiles, kPostThreads, 0, s>>>(c->r[k], n, d_tile);
    k_post_scan_tiles<<<1, 1024, 0, s>>>(d_tile, ntiles, d_total);
    const double dM = c->p.M_total / (double)n;
    k_post_energy<<<(unsigned)ntiles, kPostThreads, 0, s>>>(c->r[k], c->vr[k], c->ell[k], n, d_tile, c->p.G, dM,
                                                            d_psi, d_E);
    c->launches += 3;
    double total = 0.0;
    e = cudaGetLastError();
    if (e == cudaSuccess && psi) e = cudaMemcpyAsync(psi, d_psi, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess && E) e = cudaMemcpyAsync(E, d_E, (size_t)n * 8, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&total, d_total, 8, cudaMemcpyDeviceToHost, s);
    cudaFreeAsync(d, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_err(c, e, "potential");
    if (psi0) *psi0 = c->p.G * dM * total;
    return NSG_OK;
}
