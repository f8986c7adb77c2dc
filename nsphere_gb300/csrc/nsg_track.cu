// nsg_track.cu -- device-side trajectory recorder: the per-step tracking of
// nsphere.c:6384-6450 (r, v_r, ell, E_rel, mu of a few particles looked up through the
// inverse map after every step) kept on the GPU, so that a step needs no host round
// trip.  One kernel of one block runs at the end of each step on the context's stream
// (and so inside the captured step graph); the slot it writes comes from a device
// counter, which makes graph replays record consecutive slots.
//
// The static potential Psi(r) of the initial halo is the closed form of the
// reference's tabulated integrals (nsphere.c:4575-4592): for a density rho ~ f(r)
// normalised to mass M within r_trunc,
//     Psi(r) = G M / m(r_trunc) * [ m(r)/r + int_r^inf 4 pi r' f(r') dr' ],
// with m(r) = int_0^r 4 pi r'^2 f dr' (same units as the integral of f).  For the
// three profiles:
//   cored  f = (1 + x^2)^-3, x = r/a:  Psi = G M / (a m(X)) * [ m(x)/x + 1 / (4 (1 + x^2)^2) ],
//          m(x) = [atan x + x (x^2 - 1) / (1 + x^2)^2] / 8,  X = r_trunc / a
//   Plummer  Psi = G M / (m(R) sqrt(r^2 + a^2)),  m(R) = (R / sqrt(R^2 + a^2))^3
//   Hernquist Psi = G M / (m(R) (r + a)),          m(R) = (R / (R + a))^2
// Each operation is one IEEE double operation (this file is compiled without FMA
// contraction), in the order the oracle's restatement uses.
#include "nsg_internal.cuh"

namespace nsg {

struct TrackDev {
    int32_t *ids = nullptr;           // [k]
    double *buf = nullptr;            // [5][k][cap]
    unsigned long long *count = nullptr;
    int k = 0, k_clamped = 0;
    int64_t cap = 0;
    nsg_psi psi{};
};

struct TrackArgs {
    const int32_t *ids;
    double *buf;
    unsigned long long *count;
    int k, k_clamped;
    int64_t cap;
    nsg_psi psi;
    double G, M;
};

// m(x)/x of the cored profile: the closed form, or its series x^2/3 - 3x^4/5 + 6x^6/7
// below x = 1e-3 (the closed form cancels there).
__device__ double cored_mx_over_x(double x)
{
    if (x < 1e-3) {
        const double t = x * x;
        return t * (1.0 / 3.0 - t * (0.6 - t * (6.0 / 7.0)));
    }
    const double u = 1.0 + x * x;
    return (atan(x) + x * (x * x - 1.0) / (u * u)) / 8.0 / x;
}

__device__ double cored_m(double x)
{
    const double u = 1.0 + x * x;
    return (atan(x) + x * (x * x - 1.0) / (u * u)) / 8.0;
}

__device__ double psi_eval(const nsg_psi &q, double G, double M, double r)
{
    if (r < q.r_lo) r = q.r_lo + 1e-10;
    else if (q.r_hi > 0.0 && r > q.r_hi) r = q.r_hi - 1e-10;
    const double a = q.a, R = q.r_trunc;
    if (q.model == NSG_PSI_PLUMMER) {
        double m = 1.0;
        if (R > 0.0) {
            const double s = R / sqrt(R * R + a * a);
            m = s * s * s;
        }
        return G * M / (m * sqrt(r * r + a * a));
    }
    if (q.model == NSG_PSI_HERNQUIST) {
        double m = 1.0;
        if (R > 0.0) {
            const double s = R / (R + a);
            m = s * s;
        }
        return G * M / (m * (r + a));
    }
    // cored: m(inf) = pi/16
    const double m = R > 0.0 ? cored_m(R / a) : 0.19634954084936207;
    const double x = r / a, u = 1.0 + x * x;
    return G * M / (a * m) * (cored_mx_over_x(x) + 0.25 / (u * u));
}

__global__ void __launch_bounds__(256) k_track(TrackArgs a, const int32_t *__restrict__ inv,
                                               const double *__restrict__ r, const double *__restrict__ v,
                                               const double *__restrict__ l, int64_t n)
{
    __shared__ unsigned long long slot;
    if (threadIdx.x == 0) slot = *a.count;
    __syncthreads();
    const unsigned long long s = slot;
    if (s < (unsigned long long)a.cap) {
        for (int t = threadIdx.x; t < a.k; t += blockDim.x) {
            const int32_t j = a.ids[t];
            const int32_t p = (j >= 0 && j < n) ? inv[j] : -1;
            double rr, vrad, ell, E, mu;
            if (p < 0 || p >= n) {
                rr = vrad = ell = E = mu = __longlong_as_double(0x7ff8000000000000ll);
            } else {
                rr = r[p];
                vrad = v[p];
                ell = l[p];
                if (t >= a.k - a.k_clamped) {
                    // low-ell group (nsphere.c:6425-6433)
                    if (rr < 0.0) rr = 0.0000000001;
                    if (a.psi.r_trunc > 0.0 && rr > a.psi.r_trunc) rr = a.psi.r_trunc;
                }
                const double w = vrad * vrad + (ell * ell) / (rr * rr);
                E = psi_eval(a.psi, a.G, a.M, rr) - 0.5 * w;
                mu = vrad / sqrt(w);
            }
            double *o = a.buf + (int64_t)t * a.cap + (int64_t)s;
            const int64_t plane = (int64_t)a.k * a.cap;
            o[0] = rr;
            o[plane] = vrad;
            o[2 * plane] = ell;
            o[3 * plane] = E;
            o[4 * plane] = mu;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *a.count = s + 1;
}

void track_free(nsg_ctx *c)
{
    if (!c->track) return;
    cudaStreamSynchronize(c->stream);
    cudaFree(c->track->ids);
    cudaFree(c->track->buf);
    cudaFree(c->track->count);
    delete c->track;
    c->track = nullptr;
}

int track_step(nsg_ctx *c)
{
    TrackDev *t = c->track;
    if (!t) return NSG_OK;
    TrackArgs a{t->ids, t->buf, t->count, t->k, t->k_clamped, t->cap, t->psi, c->p.G, c->p.M_total};
    const int s = c->cur;
    k_track<<<1, 256, 0, c->stream>>>(a, c->inv, c->r[s], c->vr[s], c->ell[s], c->n);
    c->launches += 1;
    return NSG_OK;
}

}  // namespace nsg

using namespace nsg;

extern "C" {

int nsg_track_open(nsg_ctx *c, const int32_t *ids, int k, int k_clamped, const nsg_psi *psi, int64_t capacity)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (k <= 0 || !ids || !psi || capacity <= 0 || k_clamped < 0 || k_clamped > k)
        return set_err(c, NSG_EINVAL, "bad tracking arguments");
    if (psi->model != NSG_PSI_CORED && psi->model != NSG_PSI_PLUMMER && psi->model != NSG_PSI_HERNQUIST)
        return set_err(c, NSG_EINVAL, "unknown potential model");
    if (!(psi->a > 0.0)) return set_err(c, NSG_EINVAL, "scale radius must be positive");
    if ((double)k * (double)capacity * 5.0 * 8.0 > 64e9)
        return set_err(c, NSG_EINVAL, "tracking buffer above 64 GB");
    drop_graph(c);
    track_free(c);
    TrackDev *t = new TrackDev;
    t->k = k;
    t->k_clamped = k_clamped;
    t->cap = capacity;
    t->psi = *psi;
    cudaError_t e = cudaMalloc((void **)&t->ids, (size_t)k * 4);
    if (e == cudaSuccess) e = cudaMalloc((void **)&t->buf, (size_t)k * capacity * 5 * 8);
    if (e == cudaSuccess) e = cudaMalloc((void **)&t->count, sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemcpyAsync(t->ids, ids, (size_t)k * 4, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(t->count, 0, sizeof(unsigned long long), c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    c->track = t;
    if (e != cudaSuccess) {
        track_free(c);
        return cuda_err(c, e, "tracking buffers");
    }
    return NSG_OK;
}

int nsg_track_read(nsg_ctx *c, double *out, int64_t *recorded, int64_t *steps_seen)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    if (!c->track) return set_err(c, NSG_ESTATE, "no tracking open");
    TrackDev *t = c->track;
    unsigned long long cnt = 0;
    cudaError_t e = cudaMemcpyAsync(&cnt, t->count, sizeof(cnt), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && out)
        e = cudaMemcpyAsync(out, t->buf, (size_t)t->k * t->cap * 5 * 8, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_err(c, e, "tracking read");
    if (recorded) *recorded = (int64_t)cnt < t->cap ? (int64_t)cnt : t->cap;
    if (steps_seen) *steps_seen = (int64_t)cnt;
    return NSG_OK;
}

int nsg_track_close(nsg_ctx *c)
{
    if (!c) return set_err(nullptr, NSG_EINVAL, "null context");
    drop_graph(c);
    track_free(c);
    return NSG_OK;
}

}  // extern "C"
