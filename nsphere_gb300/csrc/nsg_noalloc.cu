// nsg_noalloc.cu -- nsg_sort_device_noalloc: the radial sort by (r, id) of one halo
// of at most kNaMaxN particles held in caller-owned device columns, sorted in place,
// with every scratch buffer carved from one file-scope __device__ array so that the
// call allocates no device memory (no cudaMalloc, cudaMallocAsync, cudaFree or
// library allocator, and no context).
//
// Order: the same total order as the context sort (nsg_sort, nsg_sort_particles):
// radius keys ascending (radius_key: -0.0 == +0.0, NaN last), ties by id.  Here the
// tie order is by the signed 32-bit id and then by input position, so that ids need
// not be a permutation; for valid ids (a permutation of 0..n-1) both orders agree.
//
// Algorithm: least-significant-digit radix sort with 8-bit digits over the 96-bit
// composite (radius key, id): 4 passes over the id bytes, then 8 over the key bytes.
// Each pass is a per-tile digit histogram, one exclusive scan of the digit-major
// tile counters, and a stable scatter (tiles of 2048 positions; within a tile,
// ranks from warp match masks in position order).  The carried tag holds the id and
// the input position; after the last pass the columns are gathered by position
// into a free half of the scratch and copied back.
//
// Scratch: kNaScratchBytes = 2 x 8 MiB radius keys + 2 x 8 MiB tags + 512 KiB of
// tile counters (34,078,720 bytes).  The array is reserved on a device when this
// module is loaded there (with lazy module loading, at the first call).  Nothing in
// it has to start at zero: every histogram kernel writes all 256 x tiles counters
// that the scan and scatter of its pass read.
//
// Set-up: the first call on each device looks the array's address up with
// cudaGetSymbolAddress (which loads the module on that device) and caches it; make
// that first call before any stream capture.  The device is the current device of
// the calling thread, and `stream` must belong to it.
//
// Concurrency: all calls in one process on one device share the one scratch array,
// so calls that overlap in time (on different streams, or from different threads)
// race on it and corrupt each other's results; issue them on one stream or
// serialise them.
#include <mutex>

#include "nsg_internal.cuh"

using namespace nsg;

namespace {

constexpr int64_t kNaMaxN = int64_t(1) << 20;
constexpr int kNaThreads = 256;
constexpr int kNaRounds = 8;
constexpr int kNaTile = kNaThreads * kNaRounds;          // 2048 positions
constexpr int kNaMaxTiles = int(kNaMaxN / kNaTile);      // 512
constexpr int kNaPasses = 12;                            // 4 id bytes + 8 key bytes (even)
constexpr size_t kNaColBytes = size_t(kNaMaxN) * 8;
constexpr size_t kNaOffKey0 = 0;
constexpr size_t kNaOffKey1 = kNaOffKey0 + kNaColBytes;
constexpr size_t kNaOffTag0 = kNaOffKey1 + kNaColBytes;
constexpr size_t kNaOffTag1 = kNaOffTag0 + kNaColBytes;
constexpr size_t kNaOffCount = kNaOffTag1 + kNaColBytes;
constexpr size_t kNaScratchBytes = kNaOffCount + size_t(256) * kNaMaxTiles * 4;
constexpr int kNaMaxDevices = 64;
constexpr int kNaScanThreads = 1024;

static __device__ __align__(256) unsigned char g_na_scratch[kNaScratchBytes];

std::mutex g_na_mu;
unsigned char *g_na_base[kNaMaxDevices] = {};

__device__ __forceinline__ unsigned na_digit(uint64_t key, uint64_t tag, int pass)
{
    return pass < 4 ? unsigned(tag >> (32 + 8 * pass)) & 0xffu : unsigned(key >> (8 * (pass - 4))) & 0xffu;
}

__global__ void k_na_seed(const double *__restrict__ r, const int32_t *__restrict__ id, int n,
                          uint64_t *__restrict__ key, uint64_t *__restrict__ tag)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    key[i] = radius_key(r[i]);
    tag[i] = (uint64_t(uint32_t(id[i]) ^ 0x80000000u) << 32) | uint32_t(i);
}

__global__ void __launch_bounds__(kNaThreads) k_na_hist(const uint64_t *__restrict__ key,
                                                        const uint64_t *__restrict__ tag, int n, int pass,
                                                        int ntiles, uint32_t *__restrict__ count)
{
    __shared__ uint32_t h[256];
    const int t = threadIdx.x;
    h[t] = 0;
    __syncthreads();
    const int base = blockIdx.x * kNaTile;
    for (int k = 0; k < kNaRounds; k++) {
        const int e = base + k * kNaThreads + t;
        if (e < n) atomicAdd(&h[na_digit(key[e], tag[e], pass)], 1u);
    }
    __syncthreads();
    count[t * ntiles + blockIdx.x] = h[t];
}

// Exclusive scan of m <= 256 * kNaMaxTiles counters by one block.
__global__ void __launch_bounds__(kNaScanThreads) k_na_scan(uint32_t *__restrict__ count, int m)
{
    __shared__ uint32_t wsum[kNaScanThreads / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    const int per = (m + kNaScanThreads - 1) / kNaScanThreads;
    const int lo = min(m, t * per), hi = min(m, lo + per);
    uint32_t s = 0;
    for (int j = lo; j < hi; j++) s += count[j];
    uint32_t x = s;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t v = wsum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        wsum[lane] = v;
    }
    __syncthreads();
    uint32_t run = x - s + (w > 0 ? wsum[w - 1] : 0u);
    for (int j = lo; j < hi; j++) {
        const uint32_t c = count[j];
        count[j] = run;
        run += c;
    }
}

__global__ void __launch_bounds__(kNaThreads) k_na_scatter(const uint64_t *__restrict__ key_in,
                                                           const uint64_t *__restrict__ tag_in,
                                                           uint64_t *__restrict__ key_out,
                                                           uint64_t *__restrict__ tag_out, int n, int pass,
                                                           int ntiles, const uint32_t *__restrict__ count)
{
    constexpr int W = kNaThreads / 32;
    __shared__ uint32_t run[256];
    __shared__ uint32_t wc[W][256];
    const int t = threadIdx.x, w = t >> 5;
    run[t] = count[t * ntiles + blockIdx.x];
    for (int j = 0; j < W; j++) wc[j][t] = 0;
    __syncthreads();
    const int base = blockIdx.x * kNaTile;
    for (int k = 0; k < kNaRounds; k++) {
        const int e = base + k * kNaThreads + t;
        const bool valid = e < n;
        uint64_t kv = 0, tv = 0;
        unsigned d = 256;                       // positions past n match only each other
        if (valid) {
            kv = key_in[e];
            tv = tag_in[e];
            d = na_digit(kv, tv, pass);
        }
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned before = __popc(peers & lanemask_lt());
        if (valid && before == 0) wc[w][d] = __popc(peers);
        __syncthreads();
        if (valid) {
            uint32_t off = run[d] + before;
            for (int j = 0; j < w; j++) off += wc[j][d];
            key_out[off] = kv;
            tag_out[off] = tv;
        }
        __syncthreads();
        uint32_t s = 0;
        for (int j = 0; j < W; j++) {
            s += wc[j][t];
            wc[j][t] = 0;
        }
        run[t] += s;
        __syncthreads();
    }
}

// out_a[i] = a[pos_i], out_b[i] = b[pos_i] (b may be null), pos_i = low word of tag[i].
__global__ void k_na_gather(const double *__restrict__ a, const double *__restrict__ b,
                            const uint64_t *__restrict__ tag, int n, double *__restrict__ out_a,
                            double *__restrict__ out_b)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = uint32_t(tag[i]);
    out_a[i] = a[p];
    if (b) out_b[i] = b[p];
}

__global__ void k_na_gather_id(const int32_t *__restrict__ id, const uint64_t *__restrict__ tag, int n,
                               int32_t *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = id[uint32_t(tag[i])];
}

// Address of the scratch array on the current device.  Outside stream capture it is
// looked up on every call (cheap once the module is loaded), so a context that was
// reset or replaced since the last call -- the array may then sit at a new address --
// is followed; calls made while `s` is being captured use the address cached by the
// last call on this device, which must therefore come before the capture.
int na_scratch(cudaStream_t s, unsigned char **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "nsg_sort_device_noalloc: no current device");
    if (dev < 0 || dev >= kNaMaxDevices)
        return set_err(nullptr, NSG_EDEVICE, "nsg_sort_device_noalloc: device ordinal out of range");
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    e = cudaStreamIsCapturing(s, &cap);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "nsg_sort_device_noalloc: stream query");
    std::lock_guard<std::mutex> lock(g_na_mu);
    if (cap == cudaStreamCaptureStatusNone || !g_na_base[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_na_scratch);
        if (e != cudaSuccess) return cuda_err(nullptr, e, "nsg_sort_device_noalloc: scratch address lookup");
        g_na_base[dev] = static_cast<unsigned char *>(p);
    }
    *out = g_na_base[dev];
    return NSG_OK;
}

}  // namespace

extern "C" int nsg_sort_device_noalloc(double *d_r, double *d_vr, double *d_ell, int32_t *d_id, double *d_aux,
                                       int64_t n, void *stream)
{
    if (n < 0) return set_err(nullptr, NSG_EINVAL, "nsg_sort_device_noalloc: negative particle count");
    if (n > kNaMaxN)
        return set_err(nullptr, NSG_EINVAL,
                       "nsg_sort_device_noalloc: n exceeds the fixed scratch of 1048576 particles "
                       "(use nsg_sort or nsg_sort_particles on a context)");
    if (n > 0 && (!d_r || !d_vr || !d_ell || !d_id))
        return set_err(nullptr, NSG_EINVAL, "nsg_sort_device_noalloc: null column");
    if (n <= 1) return NSG_OK;
    // an error left by earlier work of the caller is reported as such, not as this sort's
    cudaError_t pre = cudaGetLastError();
    if (pre != cudaSuccess) return cuda_err(nullptr, pre, "nsg_sort_device_noalloc: CUDA error pending before the call");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char *base = nullptr;
    if (int rc = na_scratch(s, &base)) return rc;
    const int m = int(n);
    const int ntiles = (m + kNaTile - 1) / kNaTile;
    const int blocks = (m + 255) / 256;
    uint64_t *key[2] = {reinterpret_cast<uint64_t *>(base + kNaOffKey0),
                        reinterpret_cast<uint64_t *>(base + kNaOffKey1)};
    uint64_t *tag[2] = {reinterpret_cast<uint64_t *>(base + kNaOffTag0),
                        reinterpret_cast<uint64_t *>(base + kNaOffTag1)};
    uint32_t *count = reinterpret_cast<uint32_t *>(base + kNaOffCount);

    k_na_seed<<<blocks, 256, 0, s>>>(d_r, d_id, m, key[0], tag[0]);
    for (int pass = 0; pass < kNaPasses; pass++) {
        const int a = pass & 1;
        k_na_hist<<<ntiles, kNaThreads, 0, s>>>(key[a], tag[a], m, pass, ntiles, count);
        k_na_scan<<<1, kNaScanThreads, 0, s>>>(count, 256 * ntiles);
        k_na_scatter<<<ntiles, kNaThreads, 0, s>>>(key[a], tag[a], key[a ^ 1], tag[a ^ 1], m, pass, ntiles,
                                                   count);
    }
    // a failed launch of the sort passes leaves the caller's columns untouched: the
    // gathers and copies below, which overwrite them, are not queued
    cudaError_t le = cudaPeekAtLastError();
    if (le != cudaSuccess) return cuda_err(nullptr, cudaGetLastError(), "nsg_sort_device_noalloc: sort kernels");
    // the sorted tags are in tag[0] (even pass count); key[1] and tag[1] are free
    double *t0 = reinterpret_cast<double *>(key[1]);
    double *t1 = reinterpret_cast<double *>(tag[1]);
    const size_t b = size_t(m) * 8;
    k_na_gather<<<blocks, 256, 0, s>>>(d_r, d_vr, tag[0], m, t0, t1);
    cudaError_t e = cudaMemcpyAsync(d_r, t0, b, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_vr, t1, b, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
        k_na_gather<<<blocks, 256, 0, s>>>(d_ell, d_aux, tag[0], m, t0, t1);
        e = cudaMemcpyAsync(d_ell, t0, b, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess && d_aux) e = cudaMemcpyAsync(d_aux, t1, b, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) {
        int32_t *ti = reinterpret_cast<int32_t *>(key[1]);
        k_na_gather_id<<<blocks, 256, 0, s>>>(d_id, tag[0], m, ti);
        e = cudaMemcpyAsync(d_id, ti, size_t(m) * 4, cudaMemcpyDeviceToDevice, s);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(nullptr, e, "nsg_sort_device_noalloc");
    return NSG_OK;
}
