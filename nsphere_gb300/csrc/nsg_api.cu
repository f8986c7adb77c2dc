// nsg_api.cu -- the extern "C" entry points of libnsg (declared in include/nsg.h):
// context lifetime, device buffers, host <-> device transfer, step orchestration,
// diagnostics and profiling.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <thread>

#include "nsg_internal.cuh"

namespace nsg {

static thread_local std::string g_last_err;

int set_err(nsg_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    g_last_err = msg;
    return code;
}

int cuda_err(nsg_ctx *c, cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return set_err(c, e == cudaErrorMemoryAllocation ? NSG_ENOMEM : NSG_ECUDA, m);
}

int grid_for(nsg_ctx *c, int64_t n, int threads, int per_sm)
{
    int64_t want = (n + threads - 1) / threads;
    int64_t cap = (int64_t)c->num_sms * per_sm;
    if (want < 1) want = 1;
    return (int)(want < cap ? want : cap);
}

ProfScope::ProfScope(nsg_ctx *c_, const char *name_, double bytes_, cudaStream_t stream)
    : c(c_), name(name_), bytes(bytes_), st(stream ? stream : c_->stream)
{
    if (!c->profiling) return;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
}

ProfScope::~ProfScope()
{
    if (!c->profiling || !e0) return;
    cudaEventRecord(e1, st);
    c->ev_pool.push_back(e0);
    c->ev_pool.push_back(e1);
    // the name and bytes ride along: stats are resolved at flush time
    KernelStat ks;
    ks.name = name;
    ks.bytes = bytes;
    ks.launches = -1;  // pending marker, resolved by prof_flush
    c->stats.push_back(ks);
}

void prof_flush(nsg_ctx *c)
{
    // pending entries pair with ev_pool events in order
    std::vector<KernelStat> merged;
    size_t ev = 0;
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->side);
    for (auto &ks : c->stats) {
        if (ks.launches != -1) { merged.push_back(ks); continue; }
        float ms = 0.f;
        if (ev + 1 < c->ev_pool.size()) {
            cudaEventElapsedTime(&ms, c->ev_pool[ev], c->ev_pool[ev + 1]);
            cudaEventDestroy(c->ev_pool[ev]);
            cudaEventDestroy(c->ev_pool[ev + 1]);
        }
        ev += 2;
        bool found = false;
        for (auto &m : merged)
            if (m.name == ks.name) { m.launches += 1; m.total_ms += ms; m.bytes += ks.bytes; found = true; break; }
        if (!found) { KernelStat k2 = ks; k2.launches = 1; k2.total_ms = ms; merged.push_back(k2); }
    }
    c->ev_pool.clear();
    c->stats.swap(merged);
}

void drop_graph(nsg_ctx *c)
{
    if (c->gexec) cudaGraphExecDestroy(c->gexec);
    c->gexec = nullptr;
    c->g_failed = false;
}

// --------------------------------------------------------- small kernels

__global__ void k_ids_from_double(const double *__restrict__ src, int32_t *__restrict__ dst,
                                  int64_t n, unsigned int *bad)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        double x = src[k];
        int32_t v = -1;
        if (x >= 0.0 && x < (double)n && x == floor(x)) v = (int32_t)x;
        else atomicOr(bad, 1u);
        dst[k] = v;
    }
}

// Each id must occur exactly once: count into inv (used as scratch), then check.
__global__ void k_count_ids(const int32_t *__restrict__ id, int64_t n, int32_t *__restrict__ cnt,
                            unsigned int *bad)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int32_t j = id[k];
        if (j < 0 || j >= n) { atomicOr(bad, 1u); continue; }
        atomicAdd(&cnt[j], 1);
    }
}

// Ensembles: the particle at position p belongs to the halo whose position range
// holds p, and its id must lie in that same range.
__global__ void k_check_halo_ids(const int32_t *__restrict__ id, int64_t n, Seg sg, unsigned int *bad)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int h = seg_of(sg, k);
        if (id[k] < sg.start[h] || id[k] >= sg.start[h + 1]) atomicOr(bad, 1u);
    }
}

__global__ void k_check_counts(const int32_t *__restrict__ cnt, int64_t n, unsigned int *bad)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        if (cnt[k] != 1) atomicOr(bad, 1u);
}

__global__ void k_ids_to_double(const int32_t *__restrict__ src, double *__restrict__ dst, int64_t n)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        dst[k] = (double)src[k];
}

__global__ void k_gather_ids(const int32_t *__restrict__ ids, int k, const int32_t *__restrict__ inv,
                             const double *__restrict__ r, const double *__restrict__ v,
                             const double *__restrict__ l, int64_t n, double *__restrict__ out,
                             int32_t *__restrict__ rank)
{
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= k) return;
    int32_t j = ids[t];
    int32_t p = (j >= 0 && j < n) ? inv[j] : -1;
    rank[t] = p;
    if (p < 0) { out[3 * t] = out[3 * t + 1] = out[3 * t + 2] = __longlong_as_double(0x7ff8000000000000ll); return; }
    out[3 * t] = r[p];
    out[3 * t + 1] = v[p];
    out[3 * t + 2] = l[p];
}

__global__ void k_build_inv(const int32_t *__restrict__ id, int64_t n, int32_t *__restrict__ inv)
{
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        inv[id[k]] = (int32_t)k;
}

__global__ void k_level_hist(const int8_t *__restrict__ lv, int64_t n, unsigned long long *hist)
{
    __shared__ unsigned int h[kStatBins];
    for (int b = threadIdx.x; b < kStatBins; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        int x = lv[k];
        int b;
        if (x >= 0 && x < kMaxLevels) b = x;
        else if (x == kLevelNotConverged) b = kMaxLevels;
        else b = kMaxLevels + 1;  // Levi-Civita
        atomicAdd(&h[b], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < kStatBins; b += blockDim.x)
        if (h[b]) atomicAdd(&hist[b], (unsigned long long)h[b]);
}

__global__ void k_advance_point_mass(DevCounters *ctr, double rate_dt)
{
    ctr->point_mass += rate_dt;
}

__device__ __forceinline__ uint64_t mix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

// Compares div_rn and div_rn_lat with the hardware IEEE division on `count` generated operand
// pairs of eight classes: random normals, few-bit and all-ones mantissas, equal
// mantissas, exact products, raw bit patterns (zero/subnormal/inf/NaN), and
// exponents at the edges of the normal range.
__global__ void k_selftest_div(uint64_t seed, int64_t count, unsigned long long *out, double *first)
{
    unsigned long long fast = 0;
    const uint64_t MANT = (1ull << 52) - 1;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < count;
         k += (int64_t)gridDim.x * blockDim.x) {
        uint64_t h1 = mix64(seed ^ (uint64_t)(2 * k)), h2 = mix64(seed ^ (uint64_t)(2 * k + 1));
        uint64_t h3 = mix64(h1 ^ h2);
        int cls = (int)(k & 7);
        uint64_t ea = 1023 + (h3 & 511) - 256, eb = 1023 + ((h3 >> 9) & 511) - 256;
        uint64_t ma = h1 & MANT, mb = h2 & MANT;
        if (cls == 1) mb &= ~((1ull << 40) - 1);
        if (cls == 2) { ma |= MANT ^ 0xff; mb = h2 & 0xff; }
        if (cls == 3) ma = mb;
        if (cls == 6) { ea = (h3 >> 20) & 2047; eb = (h3 >> 31) & 2047; }
        if (cls == 7) { ea = (h3 & 1) ? 1 + (h3 >> 40 & 63) : 2046 - (h3 >> 40 & 63); }
        uint64_t ua = ((h3 >> 62) << 63) | (ea << 52) | ma, ub = (eb << 52) | mb;
        double a = __longlong_as_double((long long)ua), b = __longlong_as_double((long long)ub);
        if (cls == 4) a = __dmul_rn(b, (double)((h1 >> 40) + 1));
        if (cls == 5) { a = __longlong_as_double((long long)(h1 >> 1)); b = __longlong_as_double((long long)(h2 >> 1)); }
        double q;
        bool f = div_rn_fast(a, b, &q);
        if (!f) q = __ddiv_rn(a, b);
        double t = __ddiv_rn(a, b);
        fast += f;
        bool same = (__double_as_longlong(q) == __double_as_longlong(t)) || (q != q && t != t);
        // signed zero dividends (the innermost particle's gravity numerator)
        const double z = (h1 & 1) ? -0.0 : 0.0;
        const double zq = div_rn(z, b), zh = div_rn_hw(z, b), zt = __ddiv_rn(z, b);
        same = same && ((__double_as_longlong(zq) == __double_as_longlong(zt)) || (zq != zq && zt != zt));
        same = same && ((__double_as_longlong(zh) == __double_as_longlong(zt)) || (zh != zh && zt != zt));
        // the latency-oriented division, where it claims its result
        bool ok_l, ok_z;
        const double ql = div_rn_lat(a, b, ok_l), zl = div_rn_lat(z, b, ok_z);
        if (ok_l) same = same && (__double_as_longlong(ql) == __double_as_longlong(t));
        if (ok_z) same = same && (__double_as_longlong(zl) == __double_as_longlong(zt));
        // the comparison RN(x/y) < tol without division, for tolerances at the quotient,
        // one ulp either side of it, and at a random normal number
        {
            const double x = fabs(a), y = fabs(b), qt = __ddiv_rn(x, y);
            const long long bq = __double_as_longlong(qt);
            double tol;
            switch ((h3 >> 50) & 3) {
            case 0: tol = qt; break;
            case 1: tol = __longlong_as_double(bq + 1); break;
            case 2: tol = __longlong_as_double(bq - 1); break;
            default: tol = __longlong_as_double((long long)((h1 ^ h2) & 0x7fefffffffffffffull)); break;
            }
            const RatioBound rb = ratio_bound(tol);
            bool dec;
            const bool lt = ratio_lt(x, y, rb, dec);
            if (dec) same = same && (lt == (qt < tol));
        }
        if (!same && atomicAdd(&out[1], 1ull) == 0) { first[0] = a; first[1] = b; }
    }
    atomicAdd(&out[2], fast);
}

}  // namespace nsg

using namespace nsg;

// ------------------------------------------------------------------ memory

static void free_buffers(nsg_ctx *c)
{
    auto f = [](auto *&p) { if (p) cudaFree((void *)p); p = nullptr; };
    for (int b = 0; b < 2; b++) {
        f(c->r[b]); f(c->vr[b]); f(c->ell[b]); f(c->aux[b]); f(c->id[b]);
        f(c->keys[b]); f(c->vals[b]); f(c->q_idx[b]); f(c->q_r[b]); f(c->q_v[b]);
    }
    f(c->a0); f(c->inv); f(c->level); f(c->tile_counts); f(c->digit_tot); f(c->lc_idx); f(c->lc_early);
    f(c->red_part); f(c->stage_d);
    f(c->split); f(c->bcnt); f(c->boff); f(c->bkey); f(c->bpay); f(c->bidx);
    f(c->d_seg_start); f(c->d_bbase); f(c->seg_energy);
    c->nb_cap = 0;
    c->bidx_cap = 0;
    c->bslot_cap = 0;
    c->cap = 0;
}

static int ensure_capacity(nsg_ctx *c, int64_t n)
{
    if (n <= c->cap) return NSG_OK;
    free_buffers(c);
    const size_t d8 = (size_t)n * 8, d4 = (size_t)n * 4;
    const int64_t ntiles = (n + kRadixTile - 1) / kRadixTile;
    cudaError_t e = cudaSuccess;
    // two passes over the same list: the first only adds the sizes up, so that a
    // state that cannot fit is refused before anything is allocated
    bool count_only = true;
    size_t need = 0;
    auto A = [&](auto *&p, size_t bytes) {
        bytes = bytes ? bytes : 16;
        if (count_only) { need += (bytes + 511) & ~(size_t)511; return; }
        if (e == cudaSuccess) e = cudaMalloc((void **)&p, bytes);
    };
    auto all = [&]() {
        for (int b = 0; b < 2; b++) {
            A(c->r[b], d8); A(c->vr[b], d8); A(c->ell[b], d8); A(c->id[b], d4);
            if (c->p.carry_aux) A(c->aux[b], d8);
            A(c->keys[b], d8); A(c->vals[b], d4);
            A(c->q_idx[b], d4); A(c->q_r[b], d8); A(c->q_v[b], d8);
        }
        A(c->a0, d8); A(c->inv, d4); A(c->level, (size_t)n);
        A(c->tile_counts, (size_t)ntiles * kRadixBuckets * 4); A(c->digit_tot, kRadixBuckets * 4);
        A(c->lc_idx, d4); A(c->red_part, 2 * kReduceBlocks * 8); A(c->stage_d, d8);
        A(c->lc_early, (size_t)kLcEarlyCap * 20);
    };
    all();
    size_t free_b = 0, total_b = 0;
    e = cudaMemGetInfo(&free_b, &total_b);
    if (e != cudaSuccess) return cuda_err(c, e, "device memory query");
    if (need > free_b) {
        char msg[160];
        snprintf(msg, sizeof msg, "device allocation: %lld particles need %.1f GB of device buffers, %.1f GB free",
                 (long long)n, need / 1e9, free_b / 1e9);
        return set_err(c, NSG_ENOMEM, msg);
    }
    count_only = false;
    all();
    if (e != cudaSuccess) {
        free_buffers(c);
        return cuda_err(c, e, "device allocation");
    }
    c->cap = n;
    return NSG_OK;
}

static int check_ctx(nsg_ctx *c)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    return NSG_OK;
}

static int check_params(nsg_ctx *c, const nsg_params *p)
{
    if (!p) return set_err(c, NSG_EINVAL, "null params");
    if (!(p->dt > 0.0) || !isfinite(p->dt)) return set_err(c, NSG_EINVAL, "dt must be positive and finite");
    if (p->method != NSG_METHOD_KDK && p->method != NSG_METHOD_ADAPTIVE && p->method != NSG_METHOD_ADAPTIVE_LC &&
        p->method != NSG_METHOD_FULL_LC)
        return set_err(c, NSG_EINVAL, "unknown method");
    if (p->max_subdiv < 1) return set_err(c, NSG_EINVAL, "max_subdiv must be >= 1");
    // one warp holds every level of a Levi-Civita tau-step: levels + 2 <= 32 lanes
    if (p->max_subdiv > (1LL << 29))
        return set_err(c, NSG_EINVAL, "max_subdiv above 2^29 is not supported (reference default 2^28)");
    if (p->out_type < 0 || p->out_type > 2) return set_err(c, NSG_EINVAL, "out_type must be 0, 1 or 2");
    if (p->lc_rule < 0 || p->lc_rule > 2) return set_err(c, NSG_EINVAL, "unknown lc_rule");
    if (p->max_tau_steps < 0) return set_err(c, NSG_EINVAL, "max_tau_steps must be >= 0");
    // the integrators compare against these on the integer pipe, which needs them to be numbers
    if (isnan(p->tol_r) || isnan(p->tol_v) || isnan(p->lc_radius) || isnan(p->lc_alpha))
        return set_err(c, NSG_EINVAL, "tolerances, lc_radius and lc_alpha must not be NaN");
    if (p->sched != NSG_SCHED_PLAIN && p->sched != NSG_SCHED_LEARNED) return set_err(c, NSG_EINVAL, "unknown sched");
    return NSG_OK;
}

extern "C" {

int nsg_params_default(nsg_params *p)
{
    if (!p) return set_err(nullptr, NSG_EINVAL, "null params");
    memset(p, 0, sizeof(*p));
    p->G = 1.0;
    p->M_total = 1.0;
    p->dt = 5.0e-4;
    p->tol_r = 1.0e-7;
    p->tol_v = 1.0e-7;
    p->max_subdiv = 4096LL * 4096LL * 16LL;
    p->out_type = 2;
    p->N_taumin = 10;
    p->method = NSG_METHOD_ADAPTIVE_LC;
    p->lc_rule = NSG_LC_RCRIT;
    p->lc_alpha = 0.05;
    p->lc_radius = 1.0e-3;
    p->max_tau_steps = 100000000LL;
    p->sched = NSG_SCHED_PLAIN;
    p->carry_aux = 0;
    p->sort_mode = 0;
    p->graph = 1;
    p->nonfinite_stop = 1;
    return NSG_OK;
}

// Whether the driver builds an IF conditional graph node (CUDA 12.4 and later): tried
// once on an empty graph; without it, captured steps launch the radix fallback's
// kernels directly, as eager steps do.
static bool cond_nodes_supported()
{
    cudaGraph_t g = nullptr;
    if (cudaGraphCreate(&g, 0) != cudaSuccess) { cudaGetLastError(); return false; }
    cudaGraphConditionalHandle h;
    bool ok = cudaGraphConditionalHandleCreate(&h, g, 0, 0) == cudaSuccess;
    if (ok) {
        cudaGraphNodeParams cp = {cudaGraphNodeTypeConditional};
        cp.conditional.handle = h;
        cp.conditional.type = cudaGraphCondTypeIf;
        cp.conditional.size = 1;
        cudaGraphNode_t node;
        ok = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp) == cudaSuccess;
    }
    cudaGraphDestroy(g);
    cudaGetLastError();
    return ok;
}

int nsg_create(nsg_ctx **out, const nsg_params *p, void *stream)
{
    if (!out) return set_err(nullptr, NSG_EINVAL, "null ctx pointer");
    *out = nullptr;
    if (int rc = check_params(nullptr, p)) return rc;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_err(nullptr, NSG_ECUDA, std::string("no CUDA device: ") + cudaGetErrorString(e));
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return set_err(nullptr, NSG_ECUDA, std::string("device query: ") + cudaGetErrorString(e));
    if (prop.major * 10 + prop.minor < 100)
        return set_err(nullptr, NSG_ECUDA, "libnsg is built for sm_103a (GB300); this device is sm_" +
                                               std::to_string(prop.major * 10 + prop.minor));
    nsg_ctx *c = new nsg_ctx();
    c->p = *p;
    c->device = dev;
    c->num_sms = prop.multiProcessorCount;
    if (stream) c->stream = (cudaStream_t)stream;
    else {
        e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
        c->own_stream = true;
    }
    // the leapfrog kernels run on the side stream, at the lowest priority: the
    // Levi-Civita chains on the main stream bound the step
    int prio_lo = 0, prio_hi = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&c->side, cudaStreamNonBlocking, prio_lo);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_lcsel, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_pre, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_scat, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->body, cudaStreamNonBlocking);
    // NSG_NO_CONDITIONAL_NODES=1 takes the path of drivers without conditional nodes
    // (the radix fallback launched directly inside a captured step), for tests
    if (e == cudaSuccess) {
        const char *nc = getenv("NSG_NO_CONDITIONAL_NODES");
        c->cond_nodes = cond_nodes_supported() && !(nc && nc[0] == '1');
    }
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->ctr, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMemset(c->ctr, 0, sizeof(DevCounters));
    if (e == cudaSuccess) e = cudaMallocHost((void **)&c->h_ctr, sizeof(DevCounters));
    if (e == cudaSuccess && bucket_setup(c) != NSG_OK) e = cudaErrorInvalidValue;
    if (e == cudaSuccess && fused_force_setup(c) != NSG_OK) e = cudaErrorInvalidValue;
    if (e == cudaSuccess && fused_level0_setup(c) != NSG_OK) e = cudaErrorInvalidValue;
    if (e == cudaSuccess && lc_setup(c) != NSG_OK) e = cudaErrorInvalidValue;
    if (e == cudaSuccess && p->point_mass != 0.0)
        e = cudaMemcpy(&c->ctr->point_mass, &p->point_mass, sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        int rc = cuda_err(nullptr, e, "context setup");
        nsg_destroy(c);
        return rc;
    }
    *out = c;
    return NSG_OK;
}

void nsg_destroy(nsg_ctx *c)
{
    if (!c) return;
    snap_close(c);
    track_free(c);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    for (auto ev : c->ev_pool) cudaEventDestroy(ev);
    drop_graph(c);
    free_buffers(c);
    mlp_free(c);
    if (c->ctr) cudaFree(c->ctr);
    if (c->h_ctr) cudaFreeHost(c->h_ctr);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->ev_lcsel) cudaEventDestroy(c->ev_lcsel);
    if (c->ev_pre) cudaEventDestroy(c->ev_pre);
    if (c->ev_scat) cudaEventDestroy(c->ev_scat);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->body) cudaStreamDestroy(c->body);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *nsg_last_error(nsg_ctx *c)
{
    if (c) return c->err.c_str();
    return g_last_err.c_str();
}

int nsg_set_params(nsg_ctx *c, const nsg_params *p)
{
    if (int rc = check_ctx(c)) return rc;
    if (int rc = check_params(c, p)) return rc;
    if (p->carry_aux != c->p.carry_aux && c->n > 0)
        return set_err(c, NSG_ESTATE, "carry_aux cannot change while a state is resident");
    bool pm_changed = (p->point_mass != c->p.point_mass);
    c->p = *p;
    drop_graph(c);
    if (pm_changed) {
        cudaError_t e = cudaMemcpyAsync(&c->ctr->point_mass, &c->p.point_mass, sizeof(double),
                                        cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "point mass update");
        c->sorted = false;  // a0 depends on the point mass
    }
    return NSG_OK;
}

int nsg_get_params(nsg_ctx *c, nsg_params *p)
{
    if (int rc = check_ctx(c)) return rc;
    if (!p) return set_err(c, NSG_EINVAL, "null params");
    *p = c->p;
    return NSG_OK;
}

// The checks of validate_ids, queued on the main stream (ids the kernels cannot
// convert are already -1, which the count rejects).
static int validate_ids_launch(nsg_ctx *c, const int32_t *d_id, int64_t n)
{
    // inv doubles as the count array here
    cudaError_t e = cudaMemsetAsync(c->inv, 0, (size_t)n * 4, c->stream);
    unsigned int *d_bad = &c->ctr->pad;
    if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, 4, c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "id validation setup");
    k_count_ids<<<grid_for(c, n, 256), 256, 0, c->stream>>>(d_id, n, c->inv, d_bad);
    k_check_counts<<<grid_for(c, n, 256), 256, 0, c->stream>>>(c->inv, n, d_bad);
    if (c->nseg > 1)
        k_check_halo_ids<<<grid_for(c, n, 256), 256, 0, c->stream>>>(d_id, n, seg_table(c), d_bad);
    const cudaError_t le = cudaGetLastError();
    return le == cudaSuccess ? NSG_OK : cuda_err(c, le, "id validation");
}

// Waits for the main stream and reports the checks' verdict.
static int validate_ids_finish(nsg_ctx *c, unsigned int bad_in)
{
    unsigned int *d_bad = &c->ctr->pad;
    unsigned int bad = 0;
    cudaError_t e = cudaMemcpyAsync(&c->h_ctr->pad, d_bad, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "id validation");
    bad = c->h_ctr->pad | bad_in;
    if (bad)
        return set_err(c, NSG_EIDS, c->nseg > 1 ? "particle ids must be a permutation of 0..n-1 with each "
                                                  "halo's ids in its own position range"
                                                : "particle ids must be a permutation of 0..n-1");
    return NSG_OK;
}

static int validate_ids(nsg_ctx *c, const int32_t *d_id, int64_t n, unsigned int bad_in)
{
    if (int rc = validate_ids_launch(c, d_id, n)) return rc;
    return validate_ids_finish(c, bad_in);
}

// Halo table of the resident state (one halo unless an ensemble was uploaded):
// position ranges, near-sorted buckets per halo, per-halo energy slots.
static int setup_segments(nsg_ctx *c, const int64_t *seg_n, int nseg)
{
    std::vector<int64_t> start((size_t)nseg + 1, 0);
    std::vector<int32_t> bbase((size_t)nseg + 1, 0);
    for (int h = 0; h < nseg; h++) {
        if (seg_n[h] <= 0) return set_err(c, NSG_EINVAL, "every halo needs at least one particle");
        start[h + 1] = start[h] + seg_n[h];
        const int64_t bt = (int64_t)1 << c->tune.bshift;
        bbase[h + 1] = bbase[h] + (int32_t)((seg_n[h] + bt - 1) / bt);
    }
    if (start[nseg] != c->n) return set_err(c, NSG_EINVAL, "halo sizes must add up to n");
    const int64_t nb = bbase[nseg];
    auto F = [](auto *&p) { if (p) cudaFree((void *)p); p = nullptr; };
    cudaError_t e = cudaSuccess;
    if (nb > c->nb_cap) {
        F(c->split); F(c->bcnt); F(c->boff);
        e = cudaMalloc((void **)&c->split, (size_t)nb * 8);
        // counts (two-kernel path: [nb]; fused path: nb look-back words and an overflow word)
        if (e == cudaSuccess) e = cudaMalloc((void **)&c->bcnt, (size_t)nb * 8 + 8);
        if (e == cudaSuccess) e = cudaMalloc((void **)&c->boff, (size_t)nb * 4);
        if (e != cudaSuccess) return cuda_err(c, e, "bucket buffers");
        c->nb_cap = nb;
    }
    const int64_t nbs = nb * (int64_t)bucket_cap(c);
    if (nbs > c->bslot_cap) {
        F(c->bkey); F(c->bpay);
        c->bslot_cap = 0;
        e = cudaMalloc((void **)&c->bkey, (size_t)nbs * 8);
        if (e == cudaSuccess) e = cudaMalloc((void **)&c->bpay, (size_t)nbs * 8);
        if (e != cudaSuccess) return cuda_err(c, e, "bucket slot buffers");
        c->bslot_cap = nbs;
    }
    const int64_t nbi = nb * (int64_t)fused_cap(c);
    if (nbi > c->bidx_cap) {
        F(c->bidx);
        c->bidx_cap = 0;
        e = cudaMalloc((void **)&c->bidx, (size_t)nbi * 4);
        if (e != cudaSuccess) return cuda_err(c, e, "bucket index buffer");
        c->bidx_cap = nbi;
    }
    F(c->d_seg_start); F(c->d_bbase); F(c->seg_energy);
    e = cudaMalloc((void **)&c->d_seg_start, start.size() * 8);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->d_bbase, bbase.size() * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&c->seg_energy, (size_t)2 * nseg * 8);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_seg_start, start.data(), start.size() * 8, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->d_bbase, bbase.data(), bbase.size() * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_err(c, e, "halo table");
    c->nseg = nseg;
    c->h_seg_start = start;
    c->nb_total = nb;
    return NSG_OK;
}

static int upload_common(nsg_ctx *c, int64_t n, const int64_t *seg_n = nullptr, int nseg = 1)
{
    if (n <= 0 || n > (int64_t)0x7fffffff) return set_err(c, NSG_EINVAL, "n must be in [1, 2^31-1]");
    if (nseg < 1 || nseg > 65536) return set_err(c, NSG_EINVAL, "1 to 65536 halos");
    drop_graph(c);
    // A driver that uploads every step (the reference's loop keeps its state on the
    // host) uploads a state close to the last sort's order: the splitters of that sort
    // stay usable when the halo table is the same.  Any non-decreasing splitters give a
    // correct sort -- an unrelated state only overflows buckets and takes the radix
    // fallback -- so keeping them is safe.
    const std::vector<int64_t> old_start = c->h_seg_start;
    const int64_t old_nb = c->nb_total;
    const bool old_split = c->split_valid && c->n == n;
    if (int rc = ensure_capacity(c, n)) return rc;
    c->n = n;
    const int64_t one = n;
    if (int rc = setup_segments(c, seg_n ? seg_n : &one, seg_n ? nseg : 1)) return rc;
    c->cur = 0;
    c->state_epoch++;
    c->sorted = false;
    c->inv_valid = false;
    c->split_valid = old_split && old_start == c->h_seg_start && old_nb == c->nb_total;
    return NSG_OK;
}

static int upload_host(nsg_ctx *c, const double *r, const double *vr, const double *ell,
                       const double *id_as_double, const double *aux, int64_t n, const int64_t *seg_n,
                       int nseg)
{
    if (int rc = check_ctx(c)) return rc;
    if (!r || !vr || !ell || !id_as_double) return set_err(c, NSG_EINVAL, "null column");
    if (c->p.carry_aux && !aux) return set_err(c, NSG_EINVAL, "carry_aux set but aux is null");
    if (int rc = upload_common(c, n, seg_n, nseg)) return rc;
    const size_t b = (size_t)n * 8;
    cudaStream_t s = c->stream;
    // The columns travel on three streams at once (one copy alone does not fill the
    // host link): the ids on the main stream, whose conversion starts as soon as they
    // arrive; r and ell on the side stream, v_r (and aux) on the third.  The main
    // stream waits for all of them before the ids are validated, and the validation's
    // synchronisation returns only after every copy has finished, so the caller's
    // host arrays are free again on return, as with one stream.
    cudaError_t e = cudaEventRecord(c->ev_fork, s);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->side, c->ev_fork, 0);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(c->body, c->ev_fork, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->stage_d, id_as_double, b, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->r[0], r, b, cudaMemcpyHostToDevice, c->side);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->vr[0], vr, b, cudaMemcpyHostToDevice, c->body);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->ell[0], ell, b, cudaMemcpyHostToDevice, c->side);
    if (e == cudaSuccess && c->p.carry_aux) e = cudaMemcpyAsync(c->aux[0], aux, b, cudaMemcpyHostToDevice, c->body);
    if (e == cudaSuccess) e = cudaMemsetAsync(&c->ctr->pad, 0, 4, s);
    if (e != cudaSuccess) {
        // copies already queued may still read the caller's arrays: wait for them, so
        // the arrays are free on every return, and leave no unjoined work behind
        const int rc = cuda_err(c, e, "upload copy");
        cudaStreamSynchronize(c->side);
        cudaStreamSynchronize(c->body);
        cudaStreamSynchronize(s);
        return rc;
    }
    k_ids_from_double<<<grid_for(c, n, 256), 256, 0, s>>>(c->stage_d, c->id[0], n, &c->ctr->pad);
    // the ids are checked while the other columns are still arriving
    if (int rc = validate_ids_launch(c, c->id[0], n)) {
        cudaStreamSynchronize(c->side);
        cudaStreamSynchronize(c->body);
        cudaStreamSynchronize(s);
        return rc;
    }
    e = cudaEventRecord(c->ev_join, c->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_join, 0);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev_join, c->body);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c->ev_join, 0);
    if (e != cudaSuccess) {
        const int rc = cuda_err(c, e, "upload join");
        cudaStreamSynchronize(c->side);
        cudaStreamSynchronize(c->body);
        cudaStreamSynchronize(s);
        return rc;
    }
    return validate_ids_finish(c, 0);
}

int nsg_upload(nsg_ctx *c, const double *r, const double *vr, const double *ell,
               const double *id_as_double, const double *aux, int64_t n)
{
    return upload_host(c, r, vr, ell, id_as_double, aux, n, nullptr, 1);
}

int nsg_upload_ensemble(nsg_ctx *c, const double *r, const double *vr, const double *ell,
                        const double *id_as_double, const double *aux, const int64_t *halo_n, int nhalo)
{
    if (!halo_n || nhalo < 1) return set_err(c, NSG_EINVAL, "halo sizes missing");
    int64_t n = 0;
    for (int h = 0; h < nhalo; h++) n += halo_n[h];
    return upload_host(c, r, vr, ell, id_as_double, aux, n, halo_n, nhalo);
}

int nsg_num_halos(nsg_ctx *c)
{
    return c ? c->nseg : 0;
}

int nsg_energy_halos(nsg_ctx *c, double *K, double *W)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (!c->sorted)
        if (int rc = sort_state(c)) return rc;
    if (int rc = compute_energy(c)) return rc;
    if (c->nseg <= 1) {
        cudaError_t e = cudaMemcpyAsync(c->h_ctr->energy, c->ctr->energy, 16, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "energy readback");
        if (K) K[0] = c->h_ctr->energy[0];
        if (W) W[0] = c->h_ctr->energy[1];
        return NSG_OK;
    }
    std::vector<double> h((size_t)2 * c->nseg);
    cudaError_t e = cudaMemcpyAsync(h.data(), c->seg_energy, h.size() * 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "energy readback");
    for (int k = 0; k < c->nseg; k++) {
        if (K) K[k] = h[2 * k];
        if (W) W[k] = h[2 * k + 1];
    }
    return NSG_OK;
}

int nsg_upload_particles(nsg_ctx *c, double *const *particles, int64_t n)
{
    if (!particles) return set_err(c, NSG_EINVAL, "null particles");
    return nsg_upload(c, particles[0], particles[1], particles[2], particles[3],
                      c && c->p.carry_aux ? particles[4] : nullptr, n);
}

int nsg_upload_device(nsg_ctx *c, const double *d_r, const double *d_vr, const double *d_ell,
                      const int32_t *d_id, const double *d_aux, int64_t n)
{
    if (int rc = check_ctx(c)) return rc;
    if (!d_r || !d_vr || !d_ell || !d_id) return set_err(c, NSG_EINVAL, "null column");
    if (c->p.carry_aux && !d_aux) return set_err(c, NSG_EINVAL, "carry_aux set but aux is null");
    if (int rc = upload_common(c, n)) return rc;
    const size_t b = (size_t)n * 8;
    cudaStream_t s = c->stream;
    cudaError_t e = cudaMemcpyAsync(c->r[0], d_r, b, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->vr[0], d_vr, b, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->ell[0], d_ell, b, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->id[0], d_id, (size_t)n * 4, cudaMemcpyDeviceToDevice, s);
    if (e == cudaSuccess && c->p.carry_aux) e = cudaMemcpyAsync(c->aux[0], d_aux, b, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return cuda_err(c, e, "upload copy");
    return validate_ids(c, c->id[0], n, 0);
}

int nsg_sort(nsg_ctx *c)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    return sort_state(c);
}

// One step of params.method: the reference's time-loop body (nsphere.c:5775-5838 for
// method 5, :5484-5531 for method 2).
static int one_step(nsg_ctx *c)
{
    int rc = NSG_OK;
    if (c->p.method == NSG_METHOD_KDK) {
        // the reference sorts once before its time loop (nsphere.c:5339-5342)
        if (!c->sorted) rc = sort_state(c);
        if (!rc) rc = kdk_first_half(c);
        if (!rc) rc = sort_state_kick(c);
    } else {
        rc = integrate_adaptive(c);
    }
    if (!rc) rc = track_step(c);
    if (rc) return rc;
    if (c->p.point_mass_rate != 0.0) {
        k_advance_point_mass<<<1, 1, 0, c->stream>>>(c->ctr, c->p.point_mass_rate * c->p.dt);
        c->launches += 1;
        c->p.point_mass += c->p.point_mass_rate * c->p.dt;
        c->sorted = false;
    }
    c->steps_done++;
    return NSG_OK;
}

// Captures two consecutive steps into a CUDA graph (the eager launch sequence,
// including the side-stream fork and join) and runs them once.  Returns NSG_OK
// with c->gexec set, or leaves the graph unset when capture is not possible.
static int capture_two_steps(nsg_ctx *c)
{
    const int64_t l0 = c->launches;
    const bool sorted0 = c->sorted;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) { cudaGetLastError(); c->g_failed = true; return NSG_OK; }
    int rc = one_step(c);
    if (!rc) rc = one_step(c);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(c->stream, &g);
    if (rc || e != cudaSuccess || !g) {
        if (g) cudaGraphDestroy(g);
        cudaGetLastError();
        c->g_failed = true;
        return rc ? rc : set_err(c, NSG_ECUDA, std::string("step graph capture: ") + cudaGetErrorString(e));
    }
    e = cudaGraphInstantiate(&c->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) { c->gexec = nullptr; return cuda_err(c, e, "step graph instantiate"); }
    c->g_launches = c->launches - l0;
    c->g_sorted = sorted0;
    // the captured steps' first one took the predictions made before the capture (and
    // its last one makes the next pair's) only when learned steps refresh them
    c->g_pred_refresh = (c->pred_epoch == c->state_epoch);
    e = cudaGraphLaunch(c->gexec, c->stream);
    return e == cudaSuccess ? NSG_OK : cuda_err(c, e, "step graph launch");
}

int nsg_step(nsg_ctx *c, int nsteps)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (nsteps < 0) return set_err(c, NSG_EINVAL, "nsteps must be >= 0");
    for (int j = 0; j < nsteps;) {
        // steady state: the buffers are in the parity, sort mode and sortedness a
        // captured pair of steps starts from -> replay it
        const bool graphable = c->p.graph && !c->g_failed && !c->profiling && !c->mlp_collect &&
                               nsteps - j >= 2 && c->split_valid && c->cur == 0;
        if (graphable && c->gexec && c->sorted == c->g_sorted) {
            cudaError_t e = cudaGraphLaunch(c->gexec, c->stream);
            if (e != cudaSuccess) return cuda_err(c, e, "step graph launch");
            c->launches += c->g_launches;
            c->steps_done += 2;
            c->state_epoch += 2;
            if (c->g_pred_refresh) c->pred_epoch = c->state_epoch;
            c->p.point_mass += 2 * c->p.point_mass_rate * c->p.dt;
            if (c->p.point_mass_rate != 0.0) c->sorted = false;
            j += 2;
            continue;
        }
        if (graphable && !c->gexec) {
            // a learned schedule's captured steps take the predictions the previous step
            // made: make them for the current state first
            if (c->p.sched == NSG_SCHED_LEARNED && learned_refresh(c) && c->pred_epoch != c->state_epoch) {
                const int8_t *pred = nullptr;
                if (int rc = mlp_predict_state(c, &pred, c->stream, c->cur)) return rc;
                c->pred_epoch = c->state_epoch;
            }
            if (int rc = capture_two_steps(c)) return rc;
            if (c->gexec) { j += 2; continue; }
        }
        if (int rc = one_step(c)) return rc;
        j++;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_err(c, e, "step launch");
    if (c->profiling) prof_flush(c);
    return NSG_OK;
}

int nsg_download(nsg_ctx *c, double *r, double *vr, double *ell, double *id_as_double, double *aux)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    const int s = c->cur;
    const size_t b = (size_t)c->n * 8;
    cudaStream_t st = c->stream;
    cudaError_t e = cudaSuccess;
    if (r) e = cudaMemcpyAsync(r, c->r[s], b, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && vr) e = cudaMemcpyAsync(vr, c->vr[s], b, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && ell) e = cudaMemcpyAsync(ell, c->ell[s], b, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && aux && c->p.carry_aux) e = cudaMemcpyAsync(aux, c->aux[s], b, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess && id_as_double) {
        k_ids_to_double<<<grid_for(c, c->n, 256), 256, 0, st>>>(c->id[s], c->stage_d, c->n);
        e = cudaMemcpyAsync(id_as_double, c->stage_d, b, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_err(c, e, "download");
    return NSG_OK;
}

__global__ void k_pack_lc(const unsigned int *__restrict__ cnt, const uint32_t *__restrict__ lc_idx,
                          const double *__restrict__ r, const double *__restrict__ v, uint32_t *__restrict__ oi,
                          double *__restrict__ orr, double *__restrict__ ov, unsigned int cap)
{
    const unsigned int m = *cnt < cap ? *cnt : cap;
    for (unsigned int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
        const uint32_t i = lc_idx[e];
        oi[e] = i;
        orr[e] = r[i];
        ov[e] = v[i];
    }
}

int nsg_step_download(nsg_ctx *c, int nsteps, double *r, double *vr, double *ell, double *id_as_double,
                      double *aux)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (nsteps < 1) return set_err(c, NSG_EINVAL, "nsteps must be >= 1");
    const bool lc = (c->p.method == NSG_METHOD_ADAPTIVE_LC || c->p.method == NSG_METHOD_FULL_LC) &&
                    c->p.lc_rule != NSG_LC_OFF;
    if (!lc || c->profiling) {
        if (int rc = nsg_step(c, nsteps)) return rc;
        return nsg_download(c, r, vr, ell, id_as_double, aux);
    }
    if (nsteps > 1)
        if (int rc = nsg_step(c, nsteps - 1)) return rc;
    // the last step eagerly: the side stream's leapfrog kernels are followed, in stream
    // order, by the copy of the sorted state, which then runs beside the chains
    c->gate_fallback = true;
    const int rc1 = one_step(c);
    c->gate_fallback = false;
    if (rc1) return rc1;
    const int s = c->cur;
    const size_t b = (size_t)c->n * 8;
    cudaStream_t sd = c->side;
    cudaError_t e = cudaSuccess;
    if (r) e = cudaMemcpyAsync(r, c->r[s], b, cudaMemcpyDeviceToHost, sd);
    if (e == cudaSuccess && vr) e = cudaMemcpyAsync(vr, c->vr[s], b, cudaMemcpyDeviceToHost, sd);
    if (e == cudaSuccess && ell) e = cudaMemcpyAsync(ell, c->ell[s], b, cudaMemcpyDeviceToHost, sd);
    if (e == cudaSuccess && aux && c->p.carry_aux) e = cudaMemcpyAsync(aux, c->aux[s], b, cudaMemcpyDeviceToHost, sd);
    if (e == cudaSuccess && id_as_double) {
        k_ids_to_double<<<grid_for(c, c->n, 256), 256, 0, sd>>>(c->id[s], c->stage_d, c->n);
        e = cudaMemcpyAsync(id_as_double, c->stage_d, b, cudaMemcpyDeviceToHost, sd);
    }
    if (e != cudaSuccess) return cuda_err(c, e, "step download");
    // the Levi-Civita particles' results land when the chains end: fetch them and
    // overwrite whatever the bulk copy saw at their positions
    unsigned int cnt = 0;
    e = cudaStreamSynchronize(c->stream);
    if (e == cudaSuccess) e = cudaMemcpy(&cnt, &c->ctr->lc_count, sizeof(cnt), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_err(c, e, "step download");
    std::vector<uint32_t> hi(cnt);
    std::vector<double> hr(cnt), hv(cnt);
    if (cnt > 0 && (r || vr)) {
        unsigned char *d = nullptr;
        e = cudaMallocAsync((void **)&d, (size_t)cnt * 24, c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "step download");
        uint32_t *di = reinterpret_cast<uint32_t *>(d + (size_t)cnt * 16);
        double *dr = reinterpret_cast<double *>(d), *dv = dr + cnt;
        k_pack_lc<<<(cnt + 255) / 256, 256, 0, c->stream>>>(&c->ctr->lc_count, c->lc_idx, c->r[s], c->vr[s], di, dr,
                                                           dv, cnt);
        e = cudaMemcpyAsync(hi.data(), di, (size_t)cnt * 4, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hr.data(), dr, (size_t)cnt * 8, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(hv.data(), dv, (size_t)cnt * 8, cudaMemcpyDeviceToHost, c->stream);
        cudaFreeAsync(d, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_err(c, e, "step download");
    }
    e = cudaStreamSynchronize(sd);
    if (e != cudaSuccess) return cuda_err(c, e, "step download");
    for (unsigned int k = 0; k < cnt; k++) {
        if (r) r[hi[k]] = hr[k];
        if (vr) vr[hi[k]] = hv[k];
    }
    return NSG_OK;
}

int nsg_download_particles(nsg_ctx *c, double *const *particles)
{
    if (!particles) return set_err(c, NSG_EINVAL, "null particles");
    return nsg_download(c, particles[0], particles[1], particles[2], particles[3],
                        c && c->p.carry_aux ? particles[4] : nullptr);
}

int nsg_device_state(nsg_ctx *c, double **d_r, double **d_vr, double **d_ell, int32_t **d_id, int64_t *n)
{
    if (int rc = check_ctx(c)) return rc;
    const int s = c->cur;
    if (d_r) *d_r = c->r[s];
    if (d_vr) *d_vr = c->vr[s];
    if (d_ell) *d_ell = c->ell[s];
    if (d_id) *d_id = c->id[s];
    if (n) *n = c->n;
    return NSG_OK;
}

int nsg_sort_particles(nsg_ctx *c, double *const *particles, int64_t npts)
{
    if (int rc = check_ctx(c)) return rc;
    if (int rc = nsg_upload_particles(c, particles, npts)) return rc;
    if (int rc = sort_state(c)) return rc;
    return nsg_download_particles(c, particles);
}

int nsg_gather(nsg_ctx *c, const int32_t *ids, int k, double *r, double *vr, double *ell, int32_t *rank)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (k < 0 || (k > 0 && !ids)) return set_err(c, NSG_EINVAL, "bad id list");
    if (k == 0) return NSG_OK;
    if (!c->inv_valid) {
        // no sort since the upload: map the ids of the uploaded order
        k_build_inv<<<grid_for(c, c->n, 256), 256, 0, c->stream>>>(c->id[c->cur], c->n, c->inv);
        c->inv_valid = true;
    }
    int32_t *d_ids = nullptr, *d_rank = nullptr;
    double *d_out = nullptr;
    cudaError_t e = cudaMallocAsync((void **)&d_ids, (size_t)k * 4, c->stream);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_rank, (size_t)k * 4, c->stream);
    if (e == cudaSuccess) e = cudaMallocAsync((void **)&d_out, (size_t)k * 24, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_ids, ids, (size_t)k * 4, cudaMemcpyHostToDevice, c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "gather setup");
    const int s = c->cur;
    k_gather_ids<<<(k + 127) / 128, 128, 0, c->stream>>>(d_ids, k, c->inv, c->r[s], c->vr[s], c->ell[s],
                                                         c->n, d_out, d_rank);
    std::vector<double> h((size_t)k * 3);
    std::vector<int32_t> hr((size_t)k);
    e = cudaMemcpyAsync(h.data(), d_out, (size_t)k * 24, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hr.data(), d_rank, (size_t)k * 4, cudaMemcpyDeviceToHost, c->stream);
    cudaFreeAsync(d_ids, c->stream);
    cudaFreeAsync(d_rank, c->stream);
    cudaFreeAsync(d_out, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "gather");
    for (int t = 0; t < k; t++) {
        if (r) r[t] = h[3 * t];
        if (vr) vr[t] = h[3 * t + 1];
        if (ell) ell[t] = h[3 * t + 2];
        if (rank) rank[t] = hr[t];
    }
    return NSG_OK;
}

int nsg_energy(nsg_ctx *c, double *K, double *W)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    if (!c->sorted)
        if (int rc = sort_state(c)) return rc;
    if (int rc = compute_energy(c)) return rc;
    cudaError_t e = cudaMemcpyAsync(c->h_ctr->energy, c->ctr->energy, 16, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "energy readback");
    if (K) *K = c->h_ctr->energy[0];
    if (W) *W = c->h_ctr->energy[1];
    return NSG_OK;
}

int nsg_level_hist(nsg_ctx *c, int64_t *hist, int nbins)
{
    if (int rc = check_ctx(c)) return rc;
    if (!hist || nbins < 3) return set_err(c, NSG_EINVAL, "hist needs at least 3 bins");
    if (c->n <= 0) return set_err(c, NSG_ESTATE, "no state uploaded");
    cudaError_t e = cudaMemsetAsync(c->ctr->level_hist, 0, sizeof(c->ctr->level_hist), c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "hist reset");
    k_level_hist<<<grid_for(c, c->n, 256, 4), 256, 0, c->stream>>>(c->level, c->n, c->ctr->level_hist);
    e = cudaMemcpyAsync(c->h_ctr->level_hist, c->ctr->level_hist, sizeof(c->ctr->level_hist),
                        cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "hist readback");
    for (int b = 0; b < nbins; b++) hist[b] = 0;
    for (int k = 0; k < kMaxLevels; k++) {
        int b = k < nbins - 2 ? k : nbins - 3;
        hist[b] += (int64_t)c->h_ctr->level_hist[k];
    }
    hist[nbins - 2] = (int64_t)c->h_ctr->level_hist[kMaxLevels];
    hist[nbins - 1] = (int64_t)c->h_ctr->level_hist[kMaxLevels + 1];
    return NSG_OK;
}

int nsg_levels(nsg_ctx *c, int8_t *levels)
{
    if (int rc = check_ctx(c)) return rc;
    if (!levels) return set_err(c, NSG_EINVAL, "null levels");
    cudaError_t e = cudaMemcpyAsync(levels, c->level, (size_t)c->n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "levels readback");
    return NSG_OK;
}

int nsg_sync(nsg_ctx *c, int timeout_ms)
{
    if (int rc = check_ctx(c)) return rc;
    auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        cudaError_t e = cudaStreamQuery(c->stream);
        if (e == cudaSuccess) e = cudaStreamQuery(c->side);
        if (e == cudaSuccess) break;
        if (e != cudaErrorNotReady) return cuda_err(c, e, "sync");
        if (timeout_ms >= 0 &&
            std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms))
            return set_err(c, NSG_ETIMEOUT, "nsg_sync timed out");
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    uint32_t st = 0;
    nsg_status(c, &st);
    if (st & (NSG_ST_TAU_CAP | NSG_ST_QUEUE | NSG_ST_DEVICE_WAIT))
        return set_err(c, NSG_EDEVICE, "device status word 0x" + std::to_string(st));
    return NSG_OK;
}

int nsg_status(nsg_ctx *c, uint32_t *flags)
{
    if (int rc = check_ctx(c)) return rc;
    cudaError_t e = cudaMemcpyAsync(&c->h_ctr->status, &c->ctr->status, 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "status readback");
    if (flags) *flags = c->h_ctr->status;
    return NSG_OK;
}

int nsg_clear_status(nsg_ctx *c)
{
    if (int rc = check_ctx(c)) return rc;
    cudaError_t e = cudaMemsetAsync(&c->ctr->status, 0, 4, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "status clear");
    return NSG_OK;
}

int nsg_selftest_division(uint64_t seed, int64_t count, int64_t *mismatches, int64_t *fast_path,
                          double *first_bad)
{
    if (count < 0 || !mismatches) return set_err(nullptr, NSG_EINVAL, "bad selftest arguments");
    unsigned long long *d_out = nullptr;
    double *d_first = nullptr;
    cudaError_t e = cudaMalloc((void **)&d_out, 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void **)&d_first, 2 * sizeof(double));
    if (e == cudaSuccess) e = cudaMemset(d_out, 0, 3 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(d_first, 0, 2 * sizeof(double));
    if (e == cudaSuccess) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        k_selftest_div<<<sms * 8, 256>>>(seed, count, d_out, d_first);
        e = cudaDeviceSynchronize();
    }
    unsigned long long h[3] = {0, 0, 0};
    double f[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpy(h, d_out, sizeof(h), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(f, d_first, sizeof(f), cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    cudaFree(d_first);
    if (e != cudaSuccess) return cuda_err(nullptr, e, "division selftest");
    *mismatches = (int64_t)h[1];
    if (fast_path) *fast_path = (int64_t)h[2];
    if (first_bad) { first_bad[0] = f[0]; first_bad[1] = f[1]; }
    return NSG_OK;
}

int nsg_counters(nsg_ctx *c, int64_t *launches, int64_t *steps)
{
    if (int rc = check_ctx(c)) return rc;
    if (launches) *launches = c->launches;
    if (steps) *steps = c->steps_done;
    return NSG_OK;
}

int nsg_profile(nsg_ctx *c, int enable)
{
    if (int rc = check_ctx(c)) return rc;
    if (c->profiling) prof_flush(c);
    c->profiling = enable != 0;
    c->stats.clear();
    return NSG_OK;
}

int nsg_profile_read(nsg_ctx *c, nsg_kernel_stat *stats, int max, int *count)
{
    if (int rc = check_ctx(c)) return rc;
    prof_flush(c);
    int k = 0;
    for (auto &s : c->stats) {
        if (k >= max) break;
        if (stats) {
            memset(&stats[k], 0, sizeof(nsg_kernel_stat));
            strncpy(stats[k].name, s.name.c_str(), sizeof(stats[k].name) - 1);
            stats[k].launches = s.launches;
            stats[k].total_ms = s.total_ms;
            stats[k].bytes = s.bytes;
        }
        k++;
    }
    if (count) *count = (int)c->stats.size();
    return NSG_OK;
}

}  // extern "C"

int nsg::set_halos(nsg_ctx *c, const int64_t *seg_n, int nseg)
{
    return setup_segments(c, seg_n, nseg);
}

int nsg::begin_upload(nsg_ctx *c, int64_t n)
{
    return upload_common(c, n);
}

int nsg::finish_upload_ids(nsg_ctx *c)
{
    cudaError_t e = cudaMemsetAsync(&c->ctr->pad, 0, 4, c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "id staging");
    k_ids_from_double<<<grid_for(c, c->n, 256), 256, 0, c->stream>>>(c->stage_d, c->id[0], c->n, &c->ctr->pad);
    return validate_ids(c, c->id[0], c->n, 0);
}

void nsg::build_inv(nsg_ctx *c)
{
    k_build_inv<<<grid_for(c, c->n, 256), 256, 0, c->stream>>>(c->id[c->cur], c->n, c->inv);
}
