// nsg_probe.cu -- measures the FP64 figures the roofline of the integrators uses.
//
// The measured peaks of this machine cover HBM copy bandwidth and BF16 tensor
// throughput only; the integrators are bound by the FP64 pipe (throughput) or by
// dependent FP64 latency (long serial chains).  nsg_probe_fp64 measures, on the
// current device: FP64 FMA throughput (all SMs, independent chains), IEEE double
// division throughput on the FP64 pipe and on the integer pipe (nsg_div.cuh), and
// the dependent latency of one FP64 FMA and one division for a single warp.
// nsg_probe_latency measures the dependent latencies the Levi-Civita chains are
// built around (FP64, the three divisions, integer multiply, conversions) and the
// cycles of one leading-warp substep of the Levi-Civita kernel.
#include "nsg_internal.cuh"

namespace nsg {

__global__ void k_probe_dfma(double *out, int iters, double a, double b)
{
    double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
    for (int i = 0; i < iters; i++) {
        x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
        x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}

template <bool HW>
__global__ void k_probe_div(double *out, int iters, double c)
{
    double x0 = 1.0 + threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
    for (int i = 0; i < iters; i++) {
        x0 = ddivx<HW>(c, x0 + 1.0); x1 = ddivx<HW>(c, x1 + 1.0);
        x2 = ddivx<HW>(c, x2 + 1.0); x3 = ddivx<HW>(c, x3 + 1.0);
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3;
}

// One warp, one dependent chain: cycles per operation (kind 0: FMA, 1: division).
__global__ void k_probe_latency(double *out, long long *cyc, int iters, int kind)
{
    double x = 1.5 + threadIdx.x * 1e-9;
    long long t0 = clock64();
    if (kind == 0) for (int i = 0; i < iters; i++) x = fma(x, 1.0000001, 1e-12);
    else for (int i = 0; i < iters; i++) x = __ddiv_rn(0.7, x + 1.0);
    long long t1 = clock64();
    out[threadIdx.x] = x;
    if (threadIdx.x == 0) cyc[0] = t1 - t0;
}

// Dependent-latency probes, one block on one SM, cycles per iteration from the SM
// clock.  The asm statements pin the chains between the two clock reads.
// kind: 0 DFMA chain; 1 two independent DFMA chains in one warp; 2 one DFMA chain in
// each of two warps; 3 dadd + __ddiv_rn; 4 dadd + div_rn; 5 dadd + div_rn_lat;
// 6 IMAD; 7 mul.hi.u64; 8 I2F + FMUL + F2I; 12 dadd of x and its copy from the other
// half-warp (shuffle); 13 dadd, then a 64-bit select by lane half.
__global__ void k_probe_chain(double *out, long long *cyc, int iters, int kind)
{
    const int t = threadIdx.x;
    double x = 1.5 + t * 1e-9, y = 2.5 + t * 1e-9;
    uint64_t u = 0x9E3779B97F4A7C15ull + t;
    uint32_t w = 12345u + t;
    bool ok = true;
    asm volatile("" : "+d"(x), "+d"(y), "+l"(u), "+r"(w));
    const long long t0 = clock64();
    asm volatile("" : "+d"(x), "+d"(y), "+l"(u), "+r"(w));
    switch (kind) {
    case 0: case 2:
        for (int i = 0; i < iters; i++) x = fma(x, 1.0000001, 1e-12);
        break;
    case 1:
        for (int i = 0; i < iters; i++) { x = fma(x, 1.0000001, 1e-12); y = fma(y, 0.9999999, 1e-12); }
        break;
    case 3: for (int i = 0; i < iters; i++) x = __ddiv_rn(0.7, __dadd_rn(x, 1.0)); break;
    case 4: for (int i = 0; i < iters; i++) x = div_rn(0.7, __dadd_rn(x, 1.0)); break;
    case 5: for (int i = 0; i < iters; i++) { bool o; x = div_rn_lat(0.7, __dadd_rn(x, 1.0), o); ok &= o; } break;
    case 6: for (int i = 0; i < iters; i++) asm volatile("mad.lo.u32 %0, %0, %1, %2;" : "+r"(w) : "r"(2654435761u), "r"(7u)); break;
    case 7: for (int i = 0; i < iters; i++) asm volatile("mul.hi.u64 %0, %0, %1;" : "+l"(u) : "l"(0xD1B54A32D192ED03ull)); break;
    case 12: for (int i = 0; i < iters; i++) x = __dadd_rn(x, __shfl_xor_sync(0xffffffffu, x, 16)); break;
    case 13:
        for (int i = 0; i < iters; i++) {
            const double z = __dadd_rn(x, 1e-9);
            x = (t & 16) ? x : z;
            asm volatile("" : "+d"(x));
        }
        break;
    default: for (int i = 0; i < iters; i++) w = __float2uint_rz(__uint2float_rz(w) * 0.999f) + 7u; break;
    }
    asm volatile("" : "+d"(x), "+d"(y), "+l"(u), "+r"(w));
    const long long t1 = clock64();
    out[t] = x + y + (double)(u & 1023) + (double)w + (ok ? 0.0 : 1.0);
    if (t == 0) cyc[0] = t1 - t0;
}

}  // namespace nsg

using namespace nsg;

extern "C" int nsg_probe_latency(double *cycles, int count)
{
    if (!cycles || count < 1) return set_err(nullptr, NSG_EINVAL, "latency probe needs an output array");
    double *out = nullptr;
    long long *cyc = nullptr;
    cudaError_t e = cudaMalloc((void **)&out, 64 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&cyc, sizeof(long long));
    const int n = count < 14 ? count : 14;
    for (int k = 0; k < n && e == cudaSuccess; k++) {
        long long h = 0;
        const int it = 1024;
        if (k <= 8 || k >= 12) {
            for (int rep = 0; rep < 2 && e == cudaSuccess; rep++) {
                k_probe_chain<<<1, k == 2 ? 64 : 32>>>(out, cyc, it, k);
                e = cudaDeviceSynchronize();
            }
            if (e == cudaSuccess) e = cudaMemcpy(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost);
            cycles[k] = (double)h / it;
        } else {
            double v[3] = {0.0, 0.0, 0.0};
            if (int rc = lc_probe_substep(&v[0], &v[1], &v[2])) { cudaFree(out); cudaFree(cyc); return rc; }
            cycles[k] = v[k - 9];
        }
    }
    cudaFree(out);
    cudaFree(cyc);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "latency probe");
    return NSG_OK;
}

extern "C" int nsg_probe_fp64(double *dfma_tflops, double *div_hw_gps, double *div_int_gps,
                              double *fma_latency_cycles, double *div_latency_cycles)
{
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "probe device query");
    const int blocks = sms * 8, threads = 256;
    double *out = nullptr;
    long long *cyc = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    e = cudaMalloc((void **)&out, (size_t)blocks * threads * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void **)&cyc, sizeof(long long));
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    float ms = 0.f;
    const int it = 2048;
    if (e == cudaSuccess) {
        k_probe_dfma<<<blocks, threads>>>(out, it, 1.0000001, 1e-9);
        cudaEventRecord(e0);
        k_probe_dfma<<<blocks, threads>>>(out, it, 1.0000001, 1e-9);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (dfma_tflops) *dfma_tflops = 2.0 * 8 * it * (double)blocks * threads / (ms * 1e-3) / 1e12;
    }
    if (e == cudaSuccess) {
        k_probe_div<true><<<blocks, threads>>>(out, it / 8, 0.7);
        cudaEventRecord(e0);
        k_probe_div<true><<<blocks, threads>>>(out, it / 8, 0.7);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (div_hw_gps) *div_hw_gps = 4.0 * (it / 8) * (double)blocks * threads / (ms * 1e-3) / 1e9;
    }
    if (e == cudaSuccess) {
        k_probe_div<false><<<blocks, threads>>>(out, it / 8, 0.7);
        cudaEventRecord(e0);
        k_probe_div<false><<<blocks, threads>>>(out, it / 8, 0.7);
        cudaEventRecord(e1);
        e = cudaEventSynchronize(e1);
        cudaEventElapsedTime(&ms, e0, e1);
        if (div_int_gps) *div_int_gps = 4.0 * (it / 8) * (double)blocks * threads / (ms * 1e-3) / 1e9;
    }
    for (int kind = 0; kind < 2 && e == cudaSuccess; kind++) {
        long long h = 0;
        const int li = 1024;
        k_probe_latency<<<1, 32>>>(out, cyc, li, kind);
        e = cudaDeviceSynchronize();
        if (e == cudaSuccess) e = cudaMemcpy(&h, cyc, sizeof(h), cudaMemcpyDeviceToHost);
        double v = (double)h / li;
        if (kind == 0 && fma_latency_cycles) *fma_latency_cycles = v;
        if (kind == 1 && div_latency_cycles) *div_latency_cycles = v;
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(out);
    cudaFree(cyc);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "fp64 probe");
    return NSG_OK;
}
